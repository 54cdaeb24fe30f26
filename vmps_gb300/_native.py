"""ctypes binding of the C ABI in ``include/vmps_gb300.h``.

The native library is the product: there is no Python or CPU fallback.  If
``libvmps_gb300.so`` is missing or fails to load, importing the compute entry
points raises immediately.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libvmps_gb300.so")

VMPS_OK = 0
PREC_FP64 = 0
PREC_BF16X3 = 1
PREC_TF32X3 = 2
SYM_U1 = 0
SYM_SU2 = 1
ENV_LEFT = 0
ENV_RIGHT = 1
ENV_MODES = {"FULL": 0, "TRIANGULAR": 1, "FIXED_ROWS": 2, "FIXED_COLS": 3}

ERRORS = {-1: "VMPS_E_ARG", -2: "VMPS_E_CUDA", -3: "VMPS_E_NOMEM", -4: "VMPS_E_SHAPE",
          -5: "VMPS_E_TIMEOUT", -6: "VMPS_E_NONFINITE", -7: "VMPS_E_UNSUPPORTED"}

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)


class vmps_symmetry(C.Structure):
    _fields_ = [("nq", C.c_int32), ("kind", C.c_int32 * 4)]


class vmps_blocks(C.Structure):
    _fields_ = [("nblocks", C.c_int64), ("qin", i32p), ("qout", i32p), ("qmid", i32p), ("leg", i32p),
                ("rows", i64p), ("cols", i64p), ("offset", i64p)]


class vmps_mpo_site(C.Structure):
    _fields_ = [("nnz", C.c_int64), ("s1", i32p), ("s2", i32p), ("k", i32p), ("qin", i32p), ("qout", i32p),
                ("row", i32p), ("col", i32p), ("val", f64p), ("nloc", C.c_int32), ("qloc", i32p),
                ("nop", C.c_int32), ("qop", i32p)]


class vmps_plan_stats(C.Structure):
    _fields_ = [("n_tasks", C.c_int64), ("n_chains", C.c_int64), ("n_chains_raw", C.c_int64),
                ("n_intermediates", C.c_int64), ("n_out_blocks", C.c_int64), ("n_tiles_phase1", C.c_int64),
                ("n_tiles_phase2", C.c_int64), ("flops_reference", C.c_double), ("flops_merged", C.c_double),
                ("flops_executed", C.c_double), ("flops_phase1", C.c_double), ("flops_phase2", C.c_double),
                ("bytes_algorithmic", C.c_double), ("bytes_intermediate", C.c_double),
                ("n_segments_phase2", C.c_int64), ("n_terms_phase2", C.c_int64),
                ("flops_phase2_unsummed", C.c_double),
                ("association", C.c_int32), ("reserved", C.c_int32),
                ("tensor_flops_phase1", C.c_double), ("tensor_flops_phase2", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class vmps_lanczos_stats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("refine_iterations", C.c_int32), ("hxv_fp64", C.c_int32),
                ("hxv_split", C.c_int32), ("energy_first", C.c_double), ("residual", C.c_double),
                ("ms_total", C.c_double), ("ms_wait", C.c_double), ("ms_host", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class vmps_cheb_stats(C.Structure):
    _fields_ = [("steps", C.c_int32), ("hxv", C.c_int32), ("ms_device", C.c_double), ("ms_per_step", C.c_double),
                ("ms_total", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class vmps_gmres_stats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("fp64_iterations", C.c_int32), ("outer", C.c_int32),
                ("fp64_hxv", C.c_int32), ("restarts", C.c_int32), ("reserved", C.c_int32),
                ("residual", C.c_double), ("ms_total", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class vmps_tune_info(C.Structure):
    _fields_ = [("ncap1", C.c_int32), ("ncap2", C.c_int32), ("splitk", C.c_int32), ("candidates", C.c_int32),
                ("from_cache", C.c_int32), ("reserved", C.c_int32), ("ms_default", C.c_double),
                ("ms_best", C.c_double), ("layout_key", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class vmps_split_args(C.Structure):
    _fields_ = [("nq", C.c_int32), ("n1", C.c_int32), ("n3", C.c_int32), ("n13", C.c_int32),
                ("qloc1", i32p), ("qloc3", i32p), ("pair1", i32p), ("pair3", i32p),
                ("nin", C.c_int32), ("qin", i32p), ("din", i64p), ("nout", C.c_int32), ("qout", i32p),
                ("dout", i64p), ("dmax", C.c_int64), ("eps_svd", C.c_double), ("move_right", C.c_int32),
                ("threads", C.c_int32)]


# (name, restype, argtypes)
_PROTOS = [
    ("vmps_last_error", C.c_char_p, []),
    ("vmps_version", C.c_char_p, []),
    ("vmps_ctx_create", C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    ("vmps_ctx_destroy", C.c_int, [C.c_void_p]),
    ("vmps_ctx_set_wait_budget", C.c_int, [C.c_void_p, C.c_int64]),
    ("vmps_pivot1_create", C.c_int, [C.c_void_p, C.POINTER(vmps_symmetry), C.POINTER(vmps_blocks), f64p,
                                     C.POINTER(vmps_blocks), f64p, C.POINTER(vmps_mpo_site),
                                     C.POINTER(vmps_blocks), C.POINTER(C.c_void_p)]),
    ("vmps_pivot2_create", C.c_int, [C.c_void_p, C.POINTER(vmps_symmetry), C.POINTER(vmps_blocks), f64p,
                                     C.POINTER(vmps_blocks), f64p, C.POINTER(vmps_mpo_site),
                                     C.POINTER(vmps_mpo_site), C.POINTER(vmps_blocks), C.POINTER(C.c_void_p)]),
    ("vmps_pivot0_create", C.c_int, [C.c_void_p, C.POINTER(vmps_symmetry), C.POINTER(vmps_blocks), f64p,
                                     C.POINTER(vmps_blocks), f64p, C.POINTER(vmps_blocks),
                                     C.POINTER(C.c_void_p)]),
    ("vmps_pivot1_create_terms", C.c_int, [C.c_void_p, C.POINTER(vmps_symmetry), C.c_int,
                                           C.POINTER(C.POINTER(vmps_blocks)), C.POINTER(f64p),
                                           C.POINTER(C.POINTER(vmps_blocks)), C.POINTER(f64p),
                                           C.POINTER(C.POINTER(vmps_mpo_site)), C.POINTER(vmps_blocks),
                                           C.POINTER(C.c_void_p)]),
    ("vmps_pivot2_create_terms", C.c_int, [C.c_void_p, C.POINTER(vmps_symmetry), C.c_int,
                                           C.POINTER(C.POINTER(vmps_blocks)), C.POINTER(f64p),
                                           C.POINTER(C.POINTER(vmps_blocks)), C.POINTER(f64p),
                                           C.POINTER(C.POINTER(vmps_mpo_site)), C.POINTER(C.POINTER(vmps_mpo_site)),
                                           C.POINTER(vmps_blocks), C.POINTER(C.c_void_p)]),
    ("vmps_pivot_set_penalty", C.c_int, [C.c_void_p, C.c_int, f64p, C.c_double]),
    ("vmps_pivot_autotune", C.c_int, [C.c_void_p, C.c_int, C.POINTER(vmps_tune_info)]),
    ("vmps_tune_cache_clear", C.c_int, []),
    ("vmps_pivot_set_tiling", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    ("vmps_pivot_destroy", C.c_int, [C.c_void_p]),
    ("vmps_pivot_stats", C.c_int, [C.c_void_p, C.c_int, C.POINTER(vmps_plan_stats)]),
    ("vmps_pivot_dim", C.c_int, [C.c_void_p, i64p]),
    ("vmps_pivot_chains", C.c_int, [C.c_void_p, C.c_int64, i64p, i64p, f64p, i64p]),
    ("vmps_hxv", C.c_int, [C.c_void_p, f64p, f64p, C.c_int]),
    ("vmps_hxv_multi", C.c_int, [C.c_void_p, f64p, f64p, C.c_int, C.c_int]),
    ("vmps_two_site_contract", C.c_int, [C.c_void_p, C.POINTER(vmps_symmetry), C.POINTER(vmps_blocks), f64p,
                                         C.POINTER(vmps_blocks), f64p, C.POINTER(vmps_blocks), f64p, C.c_int64,
                                         i64p]),
    ("vmps_block_products", C.c_int, [C.c_void_p, C.POINTER(vmps_symmetry), C.POINTER(vmps_blocks), f64p,
                                      C.POINTER(vmps_blocks), f64p, C.POINTER(vmps_blocks), f64p, C.c_int64, i64p,
                                      f64p]),
    ("vmps_two_site_contract_pairs", C.c_int, [C.c_void_p, C.POINTER(vmps_symmetry), C.POINTER(vmps_blocks), f64p,
                                               C.POINTER(vmps_blocks), f64p, C.POINTER(vmps_blocks), f64p, C.c_int,
                                               C.c_int, i32p]),
    ("vmps_hostla_load", C.c_int, [C.c_char_p]),
    ("vmps_two_site_split", C.c_int, [C.POINTER(vmps_split_args), C.POINTER(vmps_blocks), f64p,
                                      C.POINTER(C.c_void_p)]),
    ("vmps_two_site_split_device", C.c_int, [C.c_void_p, C.POINTER(vmps_split_args), C.POINTER(vmps_blocks), f64p,
                                             C.POINTER(C.c_void_p)]),
    ("vmps_split_info", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), i64p, i64p, i64p, i64p]),
    ("vmps_split_get", C.c_int, [C.c_void_p, i32p, i64p, i32p, i32p, i32p, i64p, i64p, f64p, i32p, i32p, i32p,
                                 i64p, i64p, f64p]),
    ("vmps_split_destroy", None, [C.c_void_p]),
    ("vmps_gauge_step", C.c_int, [C.c_int, C.c_int, C.POINTER(vmps_blocks), f64p, f64p, C.POINTER(vmps_blocks),
                                  f64p, C.c_int]),
    ("vmps_spectral_bounds", C.c_int, [C.c_void_p, f64p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("vmps_chebyshev_moments", C.c_int, [C.c_void_p, f64p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, f64p,
                                         C.POINTER(vmps_cheb_stats)]),
    ("vmps_su2_coupling_6j", C.c_int, [C.c_int64, i32p, f64p]),
    ("vmps_chebyshev_moments_parts", C.c_int, [C.c_void_p, f64p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                              C.c_int, i64p, f64p, C.POINTER(vmps_cheb_stats)]),
    ("vmps_dvec_create", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    ("vmps_dvec_destroy", C.c_int, [C.c_void_p]),
    ("vmps_dvec_upload", C.c_int, [C.c_void_p, f64p]),
    ("vmps_dvec_download", C.c_int, [C.c_void_p, f64p]),
    ("vmps_hxv_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    ("vmps_dvec_dot", C.c_int, [C.c_void_p, C.c_void_p, f64p]),
    ("vmps_dvec_axpy", C.c_int, [C.c_double, C.c_void_p, C.c_void_p]),
    ("vmps_dvec_scale", C.c_int, [C.c_void_p, C.c_double]),
    ("vmps_dvec_copy", C.c_int, [C.c_void_p, C.c_void_p]),
    ("vmps_hxv_time", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, f64p, f64p]),
    ("vmps_lanczos_ground", C.c_int, [C.c_void_p, f64p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                      f64p, C.POINTER(vmps_lanczos_stats)]),
    ("vmps_env_create", C.c_int, [C.c_void_p, C.POINTER(vmps_symmetry), C.c_int, C.POINTER(vmps_blocks),
                                  C.POINTER(vmps_blocks), C.POINTER(vmps_mpo_site), C.POINTER(vmps_blocks),
                                  C.POINTER(C.c_void_p)]),
    ("vmps_env_create_mode", C.c_int, [C.c_void_p, C.POINTER(vmps_symmetry), C.c_int, C.c_int, C.c_int64,
                                       C.c_int64, i32p, i32p, i64p, C.POINTER(vmps_blocks), C.POINTER(vmps_blocks),
                                       C.POINTER(vmps_mpo_site), C.POINTER(vmps_blocks), C.POINTER(C.c_void_p)]),
    ("vmps_env_layout", C.c_int, [C.c_void_p, i64p, i64p]),
    ("vmps_env_layout_get", C.c_int, [C.c_void_p, i32p, i32p, i32p, i32p, i64p, i64p, i64p]),
    ("vmps_env_stats", C.c_int, [C.c_void_p, C.c_int, C.POINTER(vmps_plan_stats)]),
    ("vmps_env_run", C.c_int, [C.c_void_p, f64p, f64p, f64p, f64p, C.c_int]),
    ("vmps_env_destroy", C.c_int, [C.c_void_p]),
    ("vmps_transfer_create", C.c_int, [C.c_void_p, C.POINTER(vmps_symmetry), C.c_int, C.c_int,
                                       C.POINTER(C.POINTER(vmps_blocks)), C.POINTER(f64p),
                                       C.POINTER(C.POINTER(vmps_blocks)), C.POINTER(f64p),
                                       C.POINTER(C.POINTER(vmps_mpo_site)), C.POINTER(vmps_blocks), f64p,
                                       C.c_int64, C.c_int64, i32p, i32p, i64p, C.POINTER(vmps_blocks),
                                       C.POINTER(C.c_void_p)]),
    ("vmps_transfer_hxv", C.c_int, [C.c_void_p, f64p, f64p, C.c_int]),
    ("vmps_transfer_solve", C.c_int, [C.c_void_p, f64p, f64p, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double,
                                      C.c_int, C.POINTER(vmps_gmres_stats)]),
    ("vmps_transfer_destroy", C.c_int, [C.c_void_p]),
    ("vmps_chain_fp64_noalloc", C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int32, C.c_void_p, C.c_int64,
                                          C.c_int64, C.c_void_p, C.c_int64, C.c_int64, C.c_int32, C.c_double,
                                          C.c_void_p, C.c_void_p]),
]

EXPORTED = [p[0] for p in _PROTOS]

_lib = None


class VmpsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load the native library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, res, args in _PROTOS:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != VMPS_OK:
        raise VmpsError(rc, lib().vmps_last_error().decode(errors="replace"))
