"""Equation registry: model parameters and wavefields per equation
(seistorch/eqconfigure.py:6-127).  The positional order of these lists is the
argument order of every ``_time_step`` (model params, then wavefields)."""


class Parameters:
    @staticmethod
    def valid_model_paras():
        return {"acoustic": ["vp"],
                "acoustic_habc": ["vp"],
                "acoustic_lsrtm_habc": ["vp", "m"],
                "vti_habc2": ["vp", "epsilon", "delta"],
                "acoustic_rho_habc": ["vp", "rho"],
                "vacoustic_habc": ["vp", "Q"],
                "elastic": ["vp", "vs", "rho"]}

    @staticmethod
    def secondorder_equations():
        return ["acoustic", "acoustic_habc", "acoustic_rho_habc", "vacoustic_habc", "acoustic_lsrtm_habc",
                "vti_habc2"]


class Wavefield:
    _FIELDS = {"acoustic": ["h1", "h2"],
               "acoustic_habc": ["h1", "h2"],
               "acoustic_lsrtm_habc": ["h1", "h2", "sh1", "sh2"],
               "vti_habc2": ["p1", "p2"],
               "acoustic_rho_habc": ["h1", "h2"],
               "vacoustic_habc": ["h1", "h2"],
               "elastic": ["vx", "vz", "txx", "tzz", "txz"]}

    def __init__(self, equation="acoustic"):
        if equation not in self._FIELDS:
            raise AttributeError(f"equation '{equation}' is not implemented by seistorch_gb300 "
                                 f"(available: {sorted(self._FIELDS)})")
        self.wavefields = list(self._FIELDS[equation])

    @property
    def acoustic(self):
        return list(self._FIELDS["acoustic"])

    @property
    def acoustic_habc(self):
        return list(self._FIELDS["acoustic_habc"])

    @property
    def acoustic_lsrtm_habc(self):
        return list(self._FIELDS["acoustic_lsrtm_habc"])

    @property
    def acoustic_rho_habc(self):
        return list(self._FIELDS["acoustic_rho_habc"])

    @property
    def vti_habc2(self):
        return list(self._FIELDS["vti_habc2"])

    @property
    def elastic(self):
        return list(self._FIELDS["elastic"])
