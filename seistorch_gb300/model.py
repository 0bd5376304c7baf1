"""``build_model`` (seistorch/model.py:23-94) for the native path: config ->
(cfg, WaveRNN) with the equation module imported from
``seistorch_gb300.equations2d`` (no torch.compile: the kernels are native)."""
import importlib

from .cell import WaveCell
from .config import load_config
from .eqconfigure import Parameters
from .geom import WaveGeometryFreeForm
from .rnn import WaveRNN
from .utils import set_dtype, update_cfg


def build_model(config_path, device="cuda", mode="forward", source_encoding=False, commands=None,
                logger=None, models=None):
    cfg = load_config(config_path)
    assert mode in ("forward", "inversion", "rtm"), f"unknown mode {mode}"
    set_dtype(cfg.get("dtype", "float32"))
    g = cfg["geom"]
    if g["boundary"]["type"] == "habc":
        assert "habc" in cfg["equation"], "HABC boundaries need an *_habc equation (default.py:49-51)"
    if "VEL_PATH" not in cfg:
        key = "initPath" if mode == "inversion" else "truePath"
        cfg["VEL_PATH"] = g.get(key) or {}
    if models is not None:
        first = next(iter(models.values()))
        cfg["VEL_PATH"] = {"vp": first}
    cfg = update_cfg(cfg, device=device)
    geom = WaveGeometryFreeForm(mode=mode, logger=logger, models=models, **cfg)
    geom.inversion = mode == "inversion"
    geom.to(device)
    module = importlib.import_module(f"seistorch_gb300.equations2d.{cfg['equation']}")
    fwd = module._time_step
    bwd = getattr(module, "_time_step_backward_multiple" if g.get("multiple") else "_time_step_backward", None)
    if bwd is None:
        raise ImportError(f"equation module {cfg['equation']} has no backward function")
    fwd.ACOUSTIC2nd = cfg["equation"] in Parameters.secondorder_equations()
    cell = WaveCell(geom, fwd, bwd)
    model = WaveRNN(cell, source_encoding)
    return cfg, model
