"""Build recipe and ctypes binding of librbffd_gb300.so (the C ABI in include/rbffd.h).

The library is compiled in-tree with nvcc for sm_103a only.  There is no CPU fallback:
if the shared library is missing or no CUDA device is present, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBNAME = "librbffd_gb300.so"
LIBPATH = os.path.join(BUILD, LIBNAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]

SOURCES = ["rbf_api.cu", "knn.cu", "scan.cu", "spmm.cu", "sell.cu", "algebra.cu", "stencil_build.cu", "stencil_refined_a.cu",
           "stencil_refined_b.cu", "stencil_refined_c.cu", "batched.cu", "plan.cu", "reorder.cu", "diag.cu", "mlp.cu",
           "mlp_tc.cu", "backward.cu",
           "dense.cu"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    """Compile every CUDA translation unit (in parallel) and link librbffd_gb300.so."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "rbffd.h"))
    nvcc = _nvcc()
    objs = []

    def compile_one(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if force or _stale(o, [s] + headers):
            cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, *extra_flags, "-I", INCLUDE, "-I", CSRC, "-c", s, "-o", o]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr)
        return o

    with ThreadPoolExecutor(max_workers=min(8, len(SOURCES))) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _stale(LIBPATH, objs):
        tmp = LIBPATH + f".tmp{os.getpid()}"
        cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIBPATH)
    return LIBPATH


# ---------------------------------------------------------------------- C structs
RBF_MAX_OPS = 8
# rbf_build_cfg.flags bits (include/rbffd.h)
FLAG_STENCIL_ORDER = 1
FLAG_LOCAL_UNITS = 2
FLAG_FP64_LU = 4
FLAG_NORMAL_DOF = 8


class BuildCfg(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("phs", ctypes.c_int32), ("poly_deg", ctypes.c_int32),
                ("nops", ctypes.c_int32), ("op_code", ctypes.c_int32 * RBF_MAX_OPS),
                ("op_dim", ctypes.c_int32 * RBF_MAX_OPS), ("precision", ctypes.c_int32),
                ("refine_steps", ctypes.c_int32), ("tol", ctypes.c_double), ("flags", ctypes.c_int32),
                ("seed", ctypes.c_void_p), ("sell_slice_off", ctypes.c_void_p), ("sell_col", ctypes.c_void_p),
                ("sell_val", ctypes.c_void_p), ("sell_nnz", ctypes.c_int64)]


class Hermite(ctypes.Structure):
    _fields_ = [("is_boundary", ctypes.c_void_p), ("alpha", ctypes.c_void_p), ("beta", ctypes.c_void_p),
                ("normals", ctypes.c_void_p), ("n_boundary", ctypes.c_int64)]


class BuildStats(ctypes.Structure):
    _fields_ = [("n_stencils", ctypes.c_int64), ("n_identity_rows", ctypes.c_int64),
                ("n_fallback", ctypes.c_int64), ("n_singular", ctypes.c_int64),
                ("max_residual", ctypes.c_double), ("ms_knn", ctypes.c_float),
                ("ms_build", ctypes.c_float), ("ms_total", ctypes.c_float), ("n_residuals", ctypes.c_int64),
                ("seed_rel_err_mean", ctypes.c_double)]


class Csr(ctypes.Structure):
    _fields_ = [("ne", ctypes.c_int64), ("ns", ctypes.c_int64), ("nnz", ctypes.c_int64), ("nops", ctypes.c_int32),
                ("row_ptr", ctypes.c_void_p), ("col", ctypes.c_void_p), ("val", ctypes.c_void_p)]


# exported entry points and their signatures (checked by the CPU tests against include/rbffd.h)
_P = ctypes.c_void_p
_I = ctypes.c_int
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double
SIGNATURES = {
    "rbf_version": (ctypes.c_char_p, []),
    "rbf_ctx_create": (_I, [_I, ctypes.POINTER(_P)]),
    "rbf_ctx_destroy": (_I, [_P]),
    "rbf_ctx_set_stream": (_I, [_P, _P]),
    "rbf_last_error": (ctypes.c_char_p, [_P]),
    "rbf_knn": (_I, [_P, _P, _I64, _P, _I64, _I32, _I32, _P]),
    "rbf_build_count": (_I, [_P, _I64, _I64, _I32, _P, _P, _P]),
    "rbf_build": (_I, [_P, _P, _P, _I64, _P, _I64, _P, _I32, _P, _P, _P, _P, _P, _P]),
    "rbf_build_csr": (_I, [_P, _P, _P, _I64, _P, _I64, _P, _I32, _P, _P, _P, _P]),
    "rbf_csr_free": (_I, [_P, _P]),
    "rbf_build_backward": (_I, [_P, _P, _P, _I64, _P, _I64, _P, _I32, _P, _P, _P, _P]),
    "rbf_interp_fit": (_I, [_P, _I32, _I32, _I32, _P, _I64, _P, _P]),
    "rbf_interp_eval": (_I, [_P, _I32, _I32, _I32, _P, _I64, _P, _P, _I64, _P]),
    "rbf_sytrf_rook": (_I, [_P, _I64, _P, _I64, _P, _P]),
    "rbf_sytrs_rook": (_I, [_P, _I64, _I32, _P, _I64, _P, _P, _I64]),
    "rbf_spmm": (_I, [_P, _I64, _I64, _P, _P, _P, _I32, _I32, _P, _I64, _D, _D, _P, _I64]),
    "rbf_csr_to_csc": (_I, [_P, _I64, _I64, _P, _P, _P, _P, _P, _P]),
    "rbf_weights_axpby": (_I, [_P, _I64, _D, _P, _D, _P, _P]),
    "rbf_weights_directional": (_I, [_P, _I64, _P, _I32, _P, _I64, _P, _I32, _P]),
    "rbf_sell_offsets": (_I, [_P, _I64, _P, _P, _P]),
    "rbf_sell_from_csr": (_I, [_P, _I64, _P, _P, _P, _P, _P, _P]),
    "rbf_spmv_sell": (_I, [_P, _I64, _P, _P, _P, _P, _D, _D, _P]),
    "rbf_sell_offsets_perm": (_I, [_P, _I64, _P, _P, _P, _P]),
    "rbf_sell_from_csr_perm": (_I, [_P, _I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P]),
    "rbf_spmv_sell_perm": (_I, [_P, _I64, _I64, _P, _P, _P, _P, _P, _P, _P, _D, _D, _P]),
    "rbf_spmm_noalloc": (_I, [_P, _I64, _I64, _P, _P, _P, _I32, _I32, _P, _I64, _D, _D, _P, _I64]),
    "rbf_diag_fma_peak": (_I, [_P, _I32, ctypes.POINTER(_D)]),
    "rbf_ctx_kernel_launches": (_I64, [_P]),
    "rbf_mlp_gemm": (_I, [_P, _I32, _I32, _I32, _P, _I32, _P, _I32, _P, _I32, _P, _I32, _P, _I32, _P, _I32, _P, _I32]),
    "rbf_mlp_transpose": (_I, [_P, _I32, _I32, _P, _I32, _P, _I32]),
    "rbf_build_count_ragged": (_I, [_P, _I64, _I64, _P, _P, _P, _P]),
    "rbf_build_count_normal_dof": (_I, [_P, _I64, _I64, _P, _P, _P, _P, _P]),
    "rbf_build_batched": (_I, [_P, _P, _P, _I64, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I32]),
    "rbf_tuning_report": (_I, [_P, ctypes.c_char_p, _I64]),
    "rbf_plan_create": (_I, [_P, _P, _P, _I64, _P, _I64, _P, _I32, _P, _P, _P, _I32, _P, _P, _P]),
    "rbf_plan_launch": (_I, [_P]),
    "rbf_plan_counters": (_I, [_P, _P, _P, _P]),
    "rbf_plan_destroy": (_I, [_P]),
    "rbf_reorder_points": (_I, [_P, _P, _I64, _I32, _P, _P]),
    "rbf_ctx_set_timing": (_I, [_P, _I32]),
    "rbf_ctx_last_ms": (_I, [_P, _P]),
    "rbf_mlp_gemm_tc": (_I, [_P, _I32, _I32, _I32, _P, _I32, _P, _I32, _P, _I32, _P, _P, _I32]),
    "rbf_mlp_tc_status": (_I, [_P, _P]),
    "rbf_mlp_tc_selftest_timeout": (_I, [_P, _P]),
    "rbf_mlp_features": (_I, [_P, _P, _I64, _P, _I32, _P, _I64, _I32, _P, _I32]),
    "rbf_mlp_to_bf16": (_I, [_P, _I32, _I32, _I32, _P, _I32, _P, _I32]),
    "rbf_mlp_mse": (_I, [_P, _I32, _I32, _P, _I32, _P, _I32, _P, _I32, _I32, _P]),
    "rbf_mlp_colsum": (_I, [_P, _I32, _I32, _P, _I32, _P]),
    "rbf_mlp_adam": (_I, [_P, _I64, _P, _P, _P, _P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                          _I32, _P]),
}

_lib = None
_lock = threading.Lock()


def load(path: str | None = None):
    """Load the shared library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIBPATH
        if not os.path.exists(p):
            raise RuntimeError(f"{LIBNAME} is not built ({p}); run __graft_entry__.build() or "
                               "radialbasisfunctions.jl_gb300._native.build_library()")
        L = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        return L


class RBFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


ERR = {0: "ok", -1: "argument", -2: "dimension", -3: "cuda", -4: "singular", -5: "unsupported",
       -6: "not_found", -7: "internal"}
