"""ctypes binding of libsf_gb300.so (the C ABI in include/sf_gb300.h).

The shared library is built in-tree (``strata_fdtd_gb300/_build``) by
:func:`build`, which compiles the CUDA sources for sm_103a with nvcc.  There
is no fallback: if the library is missing or no CUDA device is present, the
calls raise.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB_PATH = os.path.join(BUILD, "libsf_gb300.so")
SOURCES = ("sf_step.cu", "sf_step_march.cu", "sf_step_col.cu", "sf_step_tile.cu", "sf_step_pipe.cu",
           "sf_step_tb.cu", "sf_voxel.cu", "sf_batch.cu", "sf_adjoint.cu", "sf_api.cu")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr"]


def _nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build strata_fdtd_gb300")
    return exe


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA source (in parallel) and link libsf_gb300.so."""
    os.makedirs(BUILD, exist_ok=True)
    csrc = os.path.join(PKG, "csrc")
    include = os.path.join(ROOT, "include")
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(csrc, s))]
    deps = [os.path.join(csrc, f) for f in os.listdir(csrc)] + [
        os.path.join(include, f) for f in os.listdir(include)]
    newest = max(os.path.getmtime(d) for d in deps)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nvcc, ARCH, *NVCC_FLAGS, f"-I{include}", "-c", os.path.join(csrc, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp"
    r = subprocess.run([nvcc, ARCH, "-shared", *objs, "-o", tmp], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class SfGridDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("coeff_v", ctypes.c_float), ("coeff_p", ctypes.c_float),
                ("flags", ctypes.c_uint32)]


class SfSource(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("a", ctypes.c_int32), ("b", ctypes.c_int32),
                ("c", ctypes.c_int32)]


class SfPole(ctypes.Structure):
    _fields_ = [("material_id", ctypes.c_int32), ("kind", ctypes.c_int32),
                ("target", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("c0", ctypes.c_float), ("c1", ctypes.c_float), ("c2", ctypes.c_float),
                ("corr", ctypes.c_float), ("J", ctypes.c_void_p), ("J_prev", ctypes.c_void_p)]


class SfPlaneBC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("axis", ctypes.c_int32), ("side", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("coeff", ctypes.c_double),
                ("reflection", ctypes.c_double)]


class SfSdfNode(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("n", ctypes.c_int32), ("a", ctypes.c_double * 3),
                ("b", ctypes.c_double * 3), ("s0", ctypes.c_double), ("s1", ctypes.c_double)]


class SfDeviceInfo(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("sm_count", ctypes.c_int32),
                ("cc_major", ctypes.c_int32), ("cc_minor", ctypes.c_int32),
                ("total_mem", ctypes.c_int64), ("l2_bytes", ctypes.c_int32),
                ("max_smem_per_block", ctypes.c_int32), ("name", ctypes.c_char * 96)]


# Every exported symbol with its ctypes signature (restype, argtypes).
_P, _I, _I64, _F, _D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_double
SIGNATURES = {
    "sf_version": (ctypes.c_char_p, []),
    "sf_last_error": (ctypes.c_char_p, []),
    "sf_device_info": (_I, [_I, ctypes.POINTER(SfDeviceInfo)]),
    "sf_plan_create": (_I, [ctypes.POINTER(SfGridDesc), ctypes.POINTER(_P)]),
    "sf_plan_destroy": (_I, [_P]),
    "sf_release_deferred": (_I, []),
    "sf_plan_bind_fields": (_I, [_P] + [_P] * 8),
    "sf_plan_current": (_I, [_P]),
    "sf_plan_set_current": (_I, [_P, _I]),
    "sf_plan_set_geometry": (_I, [_P, _P, _P]),
    "sf_plan_set_pml": (_I, [_P, _P, _P, _P, _F]),
    "sf_plan_set_pml_decay": (_I, [_P, _P, _P, _P]),
    "sf_plan_set_sources": (_I, [_P, _I, _P]),
    "sf_plan_set_probes": (_I, [_P, _I, _P]),
    "sf_plan_set_ade": (_I, [_P, _P, _I, _P, _F]),
    "sf_plan_set_kernel": (_I, [_P, _I, _I]),
    "sf_plan_set_wait_limit": (_I, [_P, _I64, _I]),
    "sf_kernel_config_count": (_I, []),
    "sf_kernel_config_name": (ctypes.c_char_p, [_I]),
    "sf_plan_autotune": (_I, [_P, _I, _P, _P, _P]),
    "sf_plan_step": (_I, [_P, _I64, _P, _P, _P]),
    "sf_plan_step_ex": (_I, [_P, _I64, _P, _P, _P, _P]),
    "sf_plan_set_microphones": (_I, [_P, _I, _P, _P]),
    "sf_plan_set_microphones_ex": (_I, [_P, _I, _P, _P, _P]),
    "sf_plan_set_nonuniform": (_I, [_P, _P, _P]),
    "sf_plan_set_plane_boundaries": (_I, [_P, _I, _P]),
    "sf_plan_set_weighted_source": (_I, [_P, _I, _I64, _P, _P]),
    "sf_energy_scratch_doubles": (_I64, [_P]),
    "sf_plan_energy": (_I, [_P, _D, _D, _D, _P, _P, _P]),
    "sf_plan_energy_noalloc": (_I, [_P, _D, _D, _D, _P, _P]),
    "sf_plan_set_ade_box": (_I, [_P, _P, _P]),
    "sf_diff_coefficients": (_I, [_P, _P, _P, _P, _P, _P]),
    "sf_diff_forward": (_I, [_P, _P, _P, _P, _I, _I64, _P, _P, _P, _P]),
    "sf_diff_adjoint": (_I, [_P, _P, _P, _P, _I, _I64, _P, _P, _P, _D, _P, _P]),
    "sf_diff_grad_theta": (_I, [_P, _P, _P, _P, _P]),
    "sf_diff_grad_fields": (_I, [_P, _P, _P, _P, _P, _P]),
    "sf_batch_create": (_I, [ctypes.POINTER(_P)]),
    "sf_batch_destroy": (_I, [_P]),
    "sf_batch_add": (_I, [_P, _P, _I64, _P, _P]),
    "sf_batch_add_ex": (_I, [_P, _P, _I64, _P, _P, _P]),
    "sf_batch_clear": (_I, [_P]),
    "sf_batch_set_tiles": (_I, [_P, _I, _I]),
    "sf_batch_tiles": (_I, [_P]),
    "sf_batch_set_kernel": (_I, [_P, _I]),
    "sf_batch_autotune": (_I, [_P, _I, _P, _P, _P, _P]),
    "sf_batch_run": (_I, [_P, _I64, _I, _P]),
    "sf_voxelize": (_I, [_P, _I, _I, _I, _I, _D, _I, _P, _P]),
    "sf_voxelize_coords": (_I, [_P, _I, _I, _I, _I, _P, _I, _P, _P]),
    "sf_sdf_eval": (_I, [_P, _I, _P, _I64, _P, _P]),
    "sf_voxelize_materials": (_I, [_P, _P, _I, _P, _I, _I, _I, _D, _P, _P, _P, _P]),
}

_LIB = None


def load(path: str | None = None):
    """Load the library (build it first if it is absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or LIB_PATH
    if not os.path.exists(path):
        build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


class NativeError(RuntimeError):
    """A nonzero status from the C ABI (message from sf_last_error)."""


def check(rc: int, what: str = ""):
    if rc != 0:
        msg = load().sf_last_error().decode(errors="replace")
        raise NativeError(f"{what}: {msg}" if what else msg)
