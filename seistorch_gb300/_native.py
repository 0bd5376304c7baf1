"""Build and load ``libseistorch_gb300.so`` (the C ABI in include/seistorch_gb300.h).

The library is plain CUDA C++ compiled with nvcc for sm_103a; Python reaches it
through ctypes with raw device pointers taken from torch tensors and the
current torch CUDA stream.  There is no CPU fallback: every entry point raises
``NativeError`` when the library is missing or a call fails.
"""
import ctypes
import os
import subprocess
import sys
import threading
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(ROOT_DIR, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libseistorch_gb300.so"
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)
SOURCES = ["acoustic.cu", "acoustic_stream.cu", "acoustic_stream_fwd.cu", "acoustic_stream_bwd.cu",
           "elastic.cu", "capi.cu", "capi_elastic.cu", "capi_batch.cu", "noalloc.cu",
           "nn_gemm.cu", "nn_ops.cu", "capi_nn.cu", "habc_bwd.cu", "postproc.cu", "fft.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


class NativeError(RuntimeError):
    """A C-ABI call returned a non-zero sgb_status."""


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def build(verbose=False, force=False):
    """Compile every .cu under csrc/ in parallel and link the shared library."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = [os.path.join(BUILD_DIR, s.replace(".cu", ".o")) for s in srcs]
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "seistorch_gb300.h")]
    newest_dep = max(os.path.getmtime(d) for d in deps)

    def compile_one(src, obj):
        if not force and os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
            return
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        list(ex.map(lambda so: compile_one(*so), zip(srcs, objs)))
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


# ------------------------------------------------------------ C structs ---

c_i32 = ctypes.c_int32
c_f32 = ctypes.c_float
c_ptr = ctypes.c_void_p


class Grid(ctypes.Structure):
    _fields_ = [("nz", c_i32), ("nx", c_i32), ("pitch", c_i32), ("nshots", c_i32),
                ("dt", c_f32), ("h", c_f32)]


class Acquisition(ctypes.Structure):
    _fields_ = [("src_ptr", c_ptr), ("src_z", c_ptr), ("src_x", c_ptr), ("src_wrow", c_ptr),
                ("wavelet", c_ptr), ("nsrc", c_i32), ("nt", c_i32),
                ("rec_row_ptr", c_ptr), ("rec_x", c_ptr), ("rec_col", c_ptr),
                ("nrec", c_i32), ("nch", c_i32), ("records", c_ptr),
                ("src_zr", c_ptr), ("rec_zr", c_ptr)]


class AcousticModel(ctypes.Structure):
    _fields_ = [("order", c_i32), ("boundary", c_i32), ("habc_width", c_i32), ("multiple", c_i32),
                ("coef", c_ptr), ("vp", c_ptr), ("damp", c_ptr)]


class HabcVjpIO(ctypes.Structure):
    _fields_ = [("u", c_ptr), ("um", c_ptr), ("gy", c_ptr), ("gu", c_ptr), ("gum", c_ptr), ("gparam", c_ptr),
                ("gvp_oneway", c_ptr), ("kz", c_ptr), ("rho_c", c_ptr), ("born_m", c_ptr), ("born_u", c_ptr),
                ("born_gu", c_ptr), ("born_gm", c_ptr), ("wi_out", c_ptr)]


class BsStore(ctypes.Structure):
    _fields_ = [("iz0", c_i32), ("iz1", c_i32), ("ix0", c_i32), ("ix1", c_i32), ("ring", c_i32),
                ("ring_size", c_i32), ("ring_store", c_ptr), ("ckpt_every", c_i32),
                ("ckpt_store", c_ptr), ("habc_planes", c_ptr)]


class ElasticModel(ctypes.Structure):
    _fields_ = [("multiple", c_i32), ("coef", c_ptr)]


class ElasticIO(ctypes.Structure):
    _fields_ = [("src_fields", c_i32), ("rec_fields", c_i32 * 4), ("illum_field", c_i32)]


class BatchGroup(ctypes.Structure):
    _fields_ = [("grid", Grid), ("model", AcousticModel), ("acq", Acquisition), ("buf", c_ptr * 3),
                ("illum", c_ptr)]


class NnConv(ctypes.Structure):
    _fields_ = [("n", c_i32), ("h", c_i32), ("w", c_i32), ("cin", c_i32), ("cout", c_i32),
                ("x", c_ptr), ("wt", c_ptr), ("bias", c_ptr), ("relu", c_i32), ("mask", c_ptr),
                ("mask_cstride", c_i32), ("out_bf16", c_ptr), ("out_f32", c_ptr), ("out_cstride", c_i32),
                ("out_coff", c_i32)]


class NnWgrad(ctypes.Structure):
    _fields_ = [("n", c_i32), ("h", c_i32), ("w", c_i32), ("cin", c_i32), ("cout", c_i32),
                ("dy_chw", c_ptr), ("x_chw", c_ptr * 3), ("dw", c_ptr)]


PTR3 = c_ptr * 3
PTR2 = c_ptr * 2
PTR5 = c_ptr * 5
PTR10 = c_ptr * 10

# name -> (restype, argtypes)
SIGNATURES = {
    "sgb_version": (ctypes.c_char_p, []),
    "sgb_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "sgb_last_cuda_error": (ctypes.c_int, []),
    "sgb_device_status": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
    "sgb_set_stream_config": (ctypes.c_int, [c_i32, c_i32, c_i32]),
    "sgb_ring_size": (ctypes.c_int, [ctypes.POINTER(Grid), c_i32, c_i32, c_i32, c_i32, c_i32,
                                     ctypes.POINTER(c_i32)]),
    "sgb_acoustic_coefficients": (ctypes.c_int, [ctypes.POINTER(Grid), c_ptr, c_ptr, c_i32, c_ptr, c_ptr]),
    "sgb_acoustic_step": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel), c_ptr, c_ptr,
                                         c_ptr, c_ptr]),
    "sgb_acoustic_step_vjp": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel), c_ptr,
                                             c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr]),
    "sgb_habc_step_vjp": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel),
                                         ctypes.POINTER(HabcVjpIO), c_ptr]),
    "sgb_acoustic_forward": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel),
                                            ctypes.POINTER(Acquisition), PTR3, c_ptr, ctypes.POINTER(BsStore),
                                            ctypes.POINTER(c_i32), ctypes.POINTER(c_i32), c_ptr]),
    "sgb_acoustic_backward": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel),
                                             ctypes.POINTER(Acquisition), ctypes.POINTER(BsStore), PTR3,
                                             c_i32, c_i32, PTR3, c_ptr, c_ptr, c_ptr]),
    "sgb_acoustic_backward_noalloc": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel),
                                                     ctypes.POINTER(Acquisition), ctypes.POINTER(BsStore), PTR3,
                                                     c_i32, c_i32, c_ptr, c_ptr]),
    "sgb_vti_forward": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel),
                                       ctypes.POINTER(Acquisition), PTR3, ctypes.POINTER(BsStore),
                                       ctypes.POINTER(c_i32), ctypes.POINTER(c_i32), c_ptr]),
    "sgb_vti_backward": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel),
                                        ctypes.POINTER(Acquisition), ctypes.POINTER(BsStore), PTR3, c_i32, c_i32,
                                        PTR3, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr]),
    "sgb_vti_step": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel), c_ptr, c_ptr, c_ptr,
                                    c_ptr]),
    "sgb_rho_forward": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel), c_ptr,
                                       ctypes.POINTER(Acquisition), PTR3, ctypes.POINTER(BsStore),
                                       ctypes.POINTER(c_i32), ctypes.POINTER(c_i32), c_ptr]),
    "sgb_rho_backward": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel), c_ptr,
                                        ctypes.POINTER(Acquisition), ctypes.POINTER(BsStore), PTR3, c_i32, c_i32,
                                        PTR3, c_ptr, c_ptr, c_ptr]),
    "sgb_rho_step": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel), c_ptr, c_ptr, c_ptr,
                                    c_ptr, c_ptr]),
    "sgb_born_forward": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel), c_ptr,
                                        ctypes.POINTER(Acquisition), PTR3, PTR3, c_ptr, ctypes.POINTER(BsStore),
                                        ctypes.POINTER(c_i32), ctypes.POINTER(c_i32), c_ptr]),
    "sgb_born_step": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel), c_ptr, c_ptr, c_ptr,
                                     c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr]),
    "sgb_born_backward": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel),
                                         ctypes.POINTER(Acquisition), ctypes.POINTER(BsStore), PTR3,
                                         c_i32, c_i32, PTR3, c_ptr, c_ptr, c_ptr]),
    "sgb_acoustic_batch_forward": (ctypes.c_int, [ctypes.POINTER(BatchGroup), c_i32, ctypes.POINTER(c_i32),
                                                  ctypes.POINTER(c_i32), c_ptr]),
    "sgb_acoustic_batch_plan": (ctypes.c_int, [ctypes.POINTER(BatchGroup), c_i32, ctypes.POINTER(c_i32),
                                               ctypes.POINTER(c_i32), ctypes.POINTER(c_ptr)]),
    "sgb_plan_launch": (ctypes.c_int, [c_ptr, c_ptr]),
    "sgb_plan_destroy": (ctypes.c_int, [c_ptr]),
    "sgb_nn_conv3x3": (ctypes.c_int, [ctypes.POINTER(NnConv), c_ptr]),
    "sgb_nn_conv3x3_wgrad": (ctypes.c_int, [ctypes.POINTER(NnWgrad), c_ptr]),
    "sgb_nn_to_chw": (ctypes.c_int, [c_i32, c_i32, c_i32, c_i32, c_i32, c_i32, c_ptr, c_i32, c_ptr, c_ptr]),
    "sgb_nn_conv_in": (ctypes.c_int, [c_i32, c_i32, c_i32, c_i32, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_i32, c_ptr]),
    "sgb_nn_conv_in_wgrad": (ctypes.c_int, [c_i32, c_i32, c_i32, c_i32, c_ptr, c_ptr, c_i32, c_ptr, c_ptr,
                                            c_ptr]),
    "sgb_nn_conv_out": (ctypes.c_int, [c_i32, c_i32, c_i32, c_i32, c_ptr, c_i32, c_ptr, c_ptr, c_ptr, c_ptr]),
    "sgb_nn_conv_out_bwd": (ctypes.c_int, [c_i32, c_i32, c_i32, c_i32, c_ptr, c_ptr, c_ptr, c_i32, c_ptr, c_ptr,
                                           c_ptr, c_ptr]),
    "sgb_nn_pool2": (ctypes.c_int, [c_i32, c_i32, c_i32, c_i32, c_ptr, c_i32, c_i32, c_ptr, c_ptr]),
    "sgb_nn_up2": (ctypes.c_int, [c_i32, c_i32, c_i32, c_i32, c_ptr, c_ptr, c_i32, c_i32, c_ptr]),
    "sgb_nn_up2_bwd": (ctypes.c_int, [c_i32, c_i32, c_i32, c_i32, c_ptr, c_i32, c_i32, c_ptr, c_ptr, c_ptr]),
    "sgb_nn_pool2_bwd": (ctypes.c_int, [c_i32, c_i32, c_i32, c_i32, c_ptr, c_ptr, c_i32, c_i32, c_ptr, c_i32,
                                        c_i32, c_ptr, c_ptr]),
    "sgb_nn_bias_grad": (ctypes.c_int, [c_i32, ctypes.c_int64, c_i32, c_ptr, c_ptr, c_ptr]),
    "sgb_nn_pack_weights": (ctypes.c_int, [c_i32, c_i32, c_ptr, c_ptr, c_ptr, c_ptr]),
    "sgb_nn_adam": (ctypes.c_int, [ctypes.c_int64, c_ptr, c_ptr, c_ptr, c_ptr, c_f32, c_f32, c_f32, c_f32, c_i32,
                                   c_f32, c_ptr]),
    "sgb_nn_mse": (ctypes.c_int, [ctypes.c_int64, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr]),
    "sgb_ncg_step": (ctypes.c_int, [ctypes.c_int64, c_ptr, c_ptr, c_ptr, c_ptr, c_f32, c_i32, c_i32, c_f32, c_f32,
                                    c_ptr, c_ptr]),
    "sgb_vacoustic_work_size": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(ctypes.c_int64),
                                               ctypes.POINTER(ctypes.c_int64)]),
    "sgb_vacoustic_kterm": (ctypes.c_int, [ctypes.POINTER(Grid), c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                                           c_ptr]),
    "sgb_vacoustic_step": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel), c_ptr, c_ptr,
                                          c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr]),
    "sgb_vacoustic_forward": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(AcousticModel), c_ptr,
                                             ctypes.POINTER(Acquisition), PTR3, c_ptr, c_ptr, c_ptr,
                                             ctypes.POINTER(c_i32), ctypes.POINTER(c_i32), c_ptr]),
    "sgb_cfl_check": (ctypes.c_int, [c_i32, c_i32, c_f32, c_f32, c_f32, ctypes.POINTER(c_f32),
                                     ctypes.POINTER(c_f32)]),
    "sgb_debug_wait_probe": (ctypes.c_int, [ctypes.c_uint32, c_i32, c_ptr]),
    "sgb_l2_misfit": (ctypes.c_int, [ctypes.c_int64, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr]),
    "sgb_grad_precondition": (ctypes.c_int, [c_i32, c_i32, c_i32, c_ptr, c_ptr, c_f32, c_ptr, c_ptr, c_ptr]),
    "sgb_grad_smooth": (ctypes.c_int, [c_i32, c_i32, c_i32, c_ptr, c_i32, c_ptr, c_i32, c_i32, c_ptr, c_ptr,
                                       c_ptr]),
    "sgb_filtfilt": (ctypes.c_int, [c_i32, c_i32, c_i32, c_ptr, c_ptr, c_ptr, c_i32, c_ptr, c_ptr, c_ptr, c_ptr]),
    "sgb_sd_step": (ctypes.c_int, [ctypes.c_int64, c_ptr, c_ptr, c_f32, c_i32, c_f32, c_f32, c_ptr, c_ptr]),
    "sgb_elastic_coefficients": (ctypes.c_int, [ctypes.POINTER(Grid), c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                                                c_ptr]),
    "sgb_elastic_step": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(ElasticModel), PTR5, PTR5,
                                        c_ptr]),
    "sgb_elastic_step_vjp": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(ElasticModel), PTR2, PTR3,
                                            PTR5, PTR5, PTR3, c_ptr]),
    "sgb_elastic_forward": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(ElasticModel),
                                           ctypes.POINTER(Acquisition), ctypes.POINTER(ElasticIO), PTR10,
                                           c_ptr, ctypes.POINTER(BsStore), ctypes.POINTER(c_i32), c_ptr]),
    "sgb_elastic_backward": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(ElasticModel),
                                            ctypes.POINTER(Acquisition), ctypes.POINTER(ElasticIO),
                                            ctypes.POINTER(BsStore), PTR10, c_i32, PTR10, PTR3, c_ptr, c_ptr,
                                            c_ptr, PTR3, c_ptr]),
    "sgb_elastic_gradient": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(ElasticModel), PTR3, c_ptr,
                                            c_ptr, c_ptr, ctypes.POINTER(BsStore), c_i32, PTR3, c_ptr]),
}

_LIB = None
_LOCK = threading.Lock()


def lib_path():
    return LIB_PATH


def load(build_if_missing=True):
    """Load the shared library (building it first if needed and possible)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise NativeError(f"{LIB_NAME} is not built; run __graft_entry__.build()")
            build()
        lib = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def check(status, what):
    if status != 0:
        lib = load()
        msg = lib.sgb_status_string(status).decode()
        extra = ""
        if status == 4:
            extra = f" (cudaError {lib.sgb_last_cuda_error()})"
        raise NativeError(f"{what} failed: {msg}{extra}")


def call(name, *args):
    lib = load()
    fn = getattr(lib, name, None)
    if fn is None:
        raise NativeError(f"{LIB_NAME} does not export {name}")
    check(fn(*args), name)


SCHEME_ACOUSTIC = 0   # 2nd-order-in-time cross-stencil family (acoustic, HABC, Born, VTI, density)
SCHEME_ELASTIC = 1    # velocity-stress staggered grid


def cfl_check(scheme, order, vmax, dt, h):
    """Courant number vmax*dt/h against the scheme's stability limit (host
    only).  Returns (courant, limit); raises NativeError (CFL) above it."""
    lib = load()
    c = c_f32(0.0)
    lim = c_f32(0.0)
    st = lib.sgb_cfl_check(int(scheme), int(order), float(vmax), float(dt), float(h), ctypes.byref(c),
                           ctypes.byref(lim))
    if st == 9:
        raise NativeError(f"CFL condition violated: vmax*dt/h = {c.value:.4f} exceeds the limit {lim.value:.4f} "
                          f"of the order-{order} {'elastic' if scheme == SCHEME_ELASTIC else 'acoustic'} scheme "
                          f"(vmax {vmax:.1f} m/s, dt {dt:g} s, h {h:g} m)")
    check(st, "sgb_cfl_check")
    return c.value, lim.value


def device_status(reset=True):
    lib = load()
    out = ctypes.c_int(0)
    check(lib.sgb_device_status(ctypes.byref(out), int(reset)), "sgb_device_status")
    return out.value


def ptr(t):
    """Raw device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def stream_handle(device=None):
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
