"""On-disk formats around the hot path, with seistorch's names (io.py).

``SeisIO.read_cfg`` reads the YAML config (PyYAML when installed, else the
subset reader of ``config.py``); ``read_geom`` loads the pickled geometry
named by ``cfg['geom']['sources' / 'receivers']`` (io.py:352-364: sources
``[[x, z], ...]``, receivers ``[[[x...], [z...]], ...]``, grid indices of
the unpadded model); ``read_pkl`` / ``write_pkl``; models are ``.npy``
arrays (geom.py reads them through ``VEL_PATH``).  Shot gathers go to HDF5
as ``shot_<i>`` datasets of shape (nt, nrec, nch) (io.py:97-115) when h5py
is installed, and to ``.npy`` otherwise.
"""
import os
import pickle

import numpy as np

from . import config


class SeisIO:
    def __init__(self, cfg=None):
        self.cfg = cfg

    @staticmethod
    def path_exists(path):
        return os.path.exists(path)

    def read_cfg(self, cfg_path):
        if not self.path_exists(cfg_path):
            raise FileNotFoundError(f"Config file {cfg_path} not found.")
        return config.read_cfg(cfg_path)

    @staticmethod
    def read_pkl(path):
        with open(path, "rb") as f:
            return pickle.load(f)

    @staticmethod
    def write_pkl(path, data):
        with open(path, "wb") as f:
            pickle.dump(data, f)

    def read_geom(self, cfg=None):
        cfg = cfg if cfg is not None else self.cfg
        if cfg is None:
            raise ValueError("The configure file is not loaded.")
        spath = cfg["geom"]["sources"]
        rpath = cfg["geom"]["receivers"]
        if not os.path.exists(spath):
            raise FileNotFoundError("Cannot find the source file.")
        if not os.path.exists(rpath):
            raise FileNotFoundError("Cannot find the receiver file.")
        return self.read_pkl(spath), self.read_pkl(rpath)

    @staticmethod
    def read_model(path):
        return np.load(path, allow_pickle=False)

    @staticmethod
    def write_shots(path, shots, shot_ids=None):
        """Per-shot records (nt, nrec, nch) -> ``shot_<i>`` datasets of an HDF5
        file, or a stacked ``.npy`` when h5py is not installed (or the path
        ends in .npy)."""
        shots = [np.asarray(s, np.float32) for s in shots]
        ids = list(shot_ids) if shot_ids is not None else list(range(len(shots)))
        if not path.endswith(".npy"):
            try:
                import h5py
            except ImportError:
                h5py = None
            if h5py is not None:
                with h5py.File(path, "a") as f:
                    for i, s in zip(ids, shots):
                        key = f"shot_{i}"
                        if key in f:
                            del f[key]
                        f.create_dataset(key, data=s)
                return path
            path = os.path.splitext(path)[0] + ".npy"
        np.save(path, np.stack(shots) if len({s.shape for s in shots}) == 1 else np.array(shots, dtype=object),
                allow_pickle=True)
        return path

    @staticmethod
    def read_shot(path, shot_no):
        if path.endswith(".npy"):
            return np.load(path, allow_pickle=True)[shot_no]
        import h5py
        with h5py.File(path, "r") as f:
            return f[f"shot_{shot_no}"][...].copy()
