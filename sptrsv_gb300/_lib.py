"""ctypes binding of libsptrsv_gb300.so (the CUDA solver) and libsptrsv_gen.so (generators).

The library is the product: there is no Python or CPU fallback.  Loading fails with an
ImportError naming the missing file when the native build is absent.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsptrsv_gb300.so")
GEN_PATH = os.path.join(HERE, "libsptrsv_gen.so")

_P = np.ctypeslib.ndpointer
f64 = _P(dtype=np.float64, flags="C_CONTIGUOUS")
i64 = _P(dtype=np.int64, flags="C_CONTIGUOUS")
u64 = _P(dtype=np.uint64, flags="C_CONTIGUOUS")
i32 = _P(dtype=np.int32, flags="C_CONTIGUOUS")
f32 = _P(dtype=np.float32, flags="C_CONTIGUOUS")
c_int, c_dbl, c_sz, c_i64, c_vp = ctypes.c_int, ctypes.c_double, ctypes.c_size_t, ctypes.c_int64, ctypes.c_void_p


class Opts(ctypes.Structure):
    """struct sptrsv_opts (include/sptrsv_gb300.h)."""
    _fields_ = [("schedule", c_int), ("precision", c_int), ("rows_per_warp", c_int), ("rhs_tile", c_int),
                ("inner", c_int), ("inner_sweeps", c_int), ("max_refine", c_int), ("tol", c_dbl),
                ("spin_budget_ns", c_i64), ("resident_warps", c_int), ("inner_tol_exp", c_int)]


# C++ entry points with the reference's signatures (include/core.h, include/sptrsv_syncfree_opencl.h);
# the names are their Itanium-ABI manglings (identical on x86-64 and aarch64, where uint64_t is
# unsigned long).
DROPIN_SYMBOLS = {
    "base_gauss_lower": "_Z16base_gauss_loweriPdPmPiS_S_",
    "base_gauss_upper": "_Z16base_gauss_upperiPdPmPiS_S_i",
    "base_gauss_upper_new": "_Z20base_gauss_upper_newiPdPmPiS_S_i",
    "supernodal_upper": "_Z16supernodal_uppermPiPdS0_S_Pmii",
    "supernodal_upper_new": "_Z20supernodal_upper_newmPiPdS0_S_Pmii",
    "supernodal_blas_upper": "_Z21supernodal_blas_upperiimPiPdS0_PmS_i",
    "supernodal_blas_upper_new": "_Z25supernodal_blas_upper_newiimPiPdS0_PmS_i",
    "ccs2ccs_pad": "_Z11ccs2ccs_padPdPiPmS_S1_S0_S0_RiS2_",
    "setLevelUpAndGetMaxLevel": "_Z24setLevelUpAndGetMaxLeveliPiPmS0_",
    "barrier_upper": "_Z13barrier_upperiPdS_S_PiPmii",
    "barrier_upper_new": "_Z17barrier_upper_newiPdS_S_PiPmii",
    "sptrsv_syncfree_opencl": "_Z22sptrsv_syncfree_openclPiS_PdiiiS0_S0_i",
    "sptrsv_syncfree2_opencl": "_Z23sptrsv_syncfree2_openclPiS_PKdiiiPdS1_",
    "sptrsv_syncfree3_opencl": "_Z23sptrsv_syncfree3_openclPiS_PKdiiiPdS1_",
}

_c_int_p = ctypes.POINTER(ctypes.c_int)

DROPIN_ARGTYPES = {
    "base_gauss_lower": ([c_int, f64, u64, i32, f64, f64], c_dbl),
    "base_gauss_upper": ([c_int, f64, u64, i32, f64, f64, c_int], c_dbl),
    "base_gauss_upper_new": ([c_int, f64, u64, i32, f64, f64, c_int], c_dbl),
    "supernodal_upper": ([c_sz, i32, f64, f64, i32, u64, c_int, c_int], c_dbl),
    "supernodal_upper_new": ([c_sz, i32, f64, f64, i32, u64, c_int, c_int], c_dbl),
    "supernodal_blas_upper": ([c_int, c_int, c_sz, i32, f64, f64, u64, i32, c_int], c_dbl),
    "supernodal_blas_upper_new": ([c_int, c_int, c_sz, i32, f64, f64, u64, i32, c_int], c_dbl),
    "ccs2ccs_pad": ([f64, i32, u64, f64, u64, i32, i32, _c_int_p, _c_int_p], c_dbl),
    "setLevelUpAndGetMaxLevel": ([c_int, i32, u64, u64], c_int),
    "barrier_upper": ([c_int, f64, f64, f64, i32, u64, c_int, c_int], c_dbl),
    "barrier_upper_new": ([c_int, f64, f64, f64, i32, u64, c_int, c_int], c_dbl),
    "sptrsv_syncfree_opencl": ([i32, i32, f64, c_int, c_int, c_int, f64, f64, c_int], c_dbl),
    "sptrsv_syncfree2_opencl": ([i32, i32, f64, c_int, c_int, c_int, f64, f64], c_dbl),
    "sptrsv_syncfree3_opencl": ([i32, i32, f64, c_int, c_int, c_int, f64, f64], c_dbl),
}

# extern "C" handle API (include/sptrsv_gb300.h)
C_API = {
    "sptrsv_default_opts": ([ctypes.POINTER(Opts)], None),
    "sptrsv_status_string": ([c_int], ctypes.c_char_p),
    "sptrsv_last_status": ([], c_int),
    "sptrsv_create": ([ctypes.POINTER(c_vp), c_int], c_int),
    "sptrsv_destroy": ([c_vp], c_int),
    "sptrsv_analyse_host": ([c_vp, c_int, c_i64, i64, i32, f64], c_int),
    "sptrsv_analyse_device": ([c_vp, c_int, c_int, c_vp, c_vp, c_vp], c_int),
    "sptrsv_set_supernodes": ([c_vp, c_int, i32], c_int),
    "sptrsv_autotune": ([c_vp, c_int, ctypes.c_float, c_int, _P(dtype=np.float32, flags="C_CONTIGUOUS"), _c_int_p,
                         ctypes.POINTER(Opts)], c_int),
    "sptrsv_autotune_bounded": ([c_vp, c_int, ctypes.c_float, c_int, ctypes.c_float,
                                 _P(dtype=np.float32, flags="C_CONTIGUOUS"), i32, _c_int_p, ctypes.POINTER(Opts)],
                                c_int),
    "sptrsv_candidate": ([c_int, ctypes.POINTER(Opts)], c_int),
    "sptrsv_candidate_applicable": ([c_vp, c_int, c_int], c_int),
    "sptrsv_features": ([c_vp, c_int, _P(dtype=np.float32, flags="C_CONTIGUOUS")], c_int),
    "sptrsv_set_tuned": ([c_vp, c_int, ctypes.POINTER(Opts)], c_int),
    "sptrsv_info": ([c_vp, _c_int_p, _c_int_p, _c_int_p], c_int),
    "sptrsv_get_levels": ([c_vp, u64], c_int),
    "sptrsv_get_in_degree": ([c_vp, i32], c_int),
    "sptrsv_get_csc": ([c_vp, i32, i32, f64], c_int),
    "sptrsv_measure_fp64": ([c_int, ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)], c_int),
    "sptrsv_set_panels_mode": ([c_int], c_int),
    "sptrsv_factor_multifrontal": ([c_int, c_int, i64, i32, f64, c_int, i32, i32, c_int, ctypes.POINTER(c_vp)], c_int),
    "sptrsv_factor_info": ([c_vp, _c_int_p, ctypes.POINTER(c_i64), _c_int_p], c_int),
    "sptrsv_factor_copy": ([c_vp, i64, i32, f64, i32], c_int),
    "sptrsv_factor_device": ([c_vp, ctypes.POINTER(c_vp), ctypes.POINTER(c_vp), ctypes.POINTER(c_vp)], c_int),
    "sptrsv_factor_times": ([c_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)], c_int),
    "sptrsv_factor_free": ([c_vp], None),
    "sptrsv_get_level_buckets": ([c_vp, i32, i32], c_int),
    "sptrsv_get_level_tasks": ([c_vp, c_int, i32], c_int),
    "sptrsv_solve": ([c_vp, ctypes.POINTER(Opts), c_vp, c_vp, c_int, c_int], c_int),
    "sptrsv_solve_host": ([c_vp, ctypes.POINTER(Opts), c_vp, c_vp, c_int, c_int], c_int),
    "sptrsv_sync": ([c_vp], c_int),
    "sptrsv_last_refine": ([c_vp, _c_int_p, _c_int_p, ctypes.POINTER(c_dbl)], c_int),
    "sptrsv_device_alloc": ([c_vp, c_sz, ctypes.POINTER(c_vp)], c_int),
    "sptrsv_device_free": ([c_vp, c_vp], c_int),
    "sptrsv_host_alloc": ([c_vp, c_sz, ctypes.POINTER(c_vp)], c_int),
    "sptrsv_host_free": ([c_vp, c_vp], c_int),
    "sptrsv_copy_h2d": ([c_vp, c_vp, c_vp, c_sz], c_int),
    "sptrsv_copy_d2h": ([c_vp, c_vp, c_vp, c_sz], c_int),
    "sptrsv_timer_begin": ([c_vp], c_int),
    "sptrsv_timer_end": ([c_vp, ctypes.POINTER(ctypes.c_float)], c_int),
    "sptrsv_flush_l2": ([c_vp], c_int),
    "sptrsv_kernel_launches": ([c_vp], c_i64),
    "sptrsv_device_sm_count": ([c_vp], c_int),
    "sptrsv_solve_noalloc": ([c_int, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp], c_int),
    "sptrsv_profile_enable": ([c_vp, c_int], c_int),
    "sptrsv_profile_read": ([c_vp, i32, _P(dtype=np.float32, flags="C_CONTIGUOUS"), c_int], c_int),
    "sptrsv_batch_create": ([ctypes.POINTER(c_vp), c_int, c_int, i32, i32, i64, i32, f64], c_int),
    "sptrsv_batch_destroy": ([c_vp], c_int),
    "sptrsv_batch_get_schedule": ([c_vp, i32], c_int),
    "sptrsv_batch_set_schedule": ([c_vp, i32], c_int),
    "sptrsv_batch_set_options": ([c_vp, c_dbl, c_int, c_int, c_i64], c_int),
    "sptrsv_batch_solve": ([c_vp, c_int, c_vp, c_vp], c_int),
    "sptrsv_batch_solve_host": ([c_vp, c_int, c_vp, c_vp], c_int),
    "sptrsv_batch_sync": ([c_vp, ctypes.POINTER(c_i64)], c_int),
    "sptrsv_batch_stats": ([c_vp, i32, i32, f64, i32], c_int),
    "sptrsv_batch_info": ([c_vp, i64, _P(dtype=np.float32, flags="C_CONTIGUOUS")], c_int),
    "sptrsv_batch_features": ([c_vp, c_int, _P(dtype=np.float32, flags="C_CONTIGUOUS")], c_int),
    "sptrsv_batch_profile": ([c_vp, c_int, c_vp, c_vp, f32, i32, f32], c_int),
    "sptrsv_batch_timer_begin": ([c_vp], c_int),
    "sptrsv_batch_timer_end": ([c_vp, ctypes.POINTER(ctypes.c_float)], c_int),
    "sptrsv_batch_launches": ([c_vp], c_i64),
    "sptrsv_read_csr": ([ctypes.c_char_p, _c_int_p, ctypes.POINTER(c_i64), ctypes.POINTER(c_vp), ctypes.POINTER(c_vp),
                         ctypes.POINTER(c_vp)], c_int),
    "sptrsv_write_csr": ([ctypes.c_char_p, c_int, c_i64, i64, i32, f64], c_int),
    "sptrsv_read_snodes": ([ctypes.c_char_p, _c_int_p, ctypes.POINTER(c_vp)], c_int),
    "sptrsv_write_snodes": ([ctypes.c_char_p, c_int, i32], c_int),
    "sptrsv_io_free": ([c_vp], None),
    "sptrsv_mlp_create": ([ctypes.POINTER(c_vp), c_int, c_int, c_int, c_int, c_int, ctypes.c_uint64], c_int),
    "sptrsv_mlp_destroy": ([c_vp], c_int),
    "sptrsv_mlp_num_params": ([c_vp], c_int),
    "sptrsv_mlp_get_params": ([c_vp, f32], c_int),
    "sptrsv_mlp_set_params": ([c_vp, f32], c_int),
    "sptrsv_mlp_set_norm": ([c_vp, f32, f32], c_int),
    "sptrsv_mlp_grad": ([c_vp, c_int, f32, f32, f32, f32, f32], c_int),
    "sptrsv_mlp_train": ([c_vp, c_int, f32, f32, f32, c_int, c_int, ctypes.c_float, ctypes.c_uint64, f32], c_int),
    "sptrsv_mlp_predict": ([c_vp, c_int, f32, f32], c_int),
    "sptrsv_mlp_launches": ([c_vp], c_i64),
}

GEN_API = {
    "sptrsv_gen_laplace2d_cholesky": ([c_int], c_vp),
    "sptrsv_gen_random_upper": ([c_int, c_dbl, c_dbl, c_int, ctypes.c_uint64], c_vp),
    "sptrsv_gen_n": ([c_vp], c_int),
    "sptrsv_gen_nnz": ([c_vp], c_i64),
    "sptrsv_gen_copy": ([c_vp, i64, i32, f64], None),
    "sptrsv_gen_free": ([c_vp], None),
    "sptrsv_gen_uniform": ([ctypes.c_uint64, c_i64, c_dbl, c_dbl, f64], None),
    "sptrsv_gen_spmv": ([c_int, i64, i32, f64, f64, f64, c_int], None),
    "sptrsv_gen_supernodal_random": ([c_int, c_int, c_int, c_dbl, c_dbl, c_int, ctypes.c_uint64,
                                      ctypes.POINTER(ctypes.POINTER(c_int)), ctypes.POINTER(c_int)], c_vp),
    "sptrsv_gen_free_ints": ([c_vp], None),
    "sptrsv_gen_mix": ([c_int, ctypes.c_uint64, c_int, c_int, c_dbl, c_dbl, c_int, c_int], c_vp),
    "sptrsv_gen_mix_array": ([c_vp, c_int, ctypes.POINTER(c_vp), ctypes.POINTER(c_i64)], c_int),
    "sptrsv_gen_mix_free": ([c_vp], None),
}

_lib = None
_gen = None


def _bind(lib, table):
    for name, (args, res) in table.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


def lib():
    """The CUDA solver library (loads it on first use; raises ImportError when unbuilt)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libsptrsv_gb300.so is not built (run __graft_entry__.build() or "
                              "python sptrsv_gb300/build.py): " + LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        _bind(L, C_API)
        for name, mangled in DROPIN_SYMBOLS.items():
            fn = getattr(L, mangled)
            fn.argtypes, fn.restype = DROPIN_ARGTYPES[name]
        _lib = L
    return _lib


def dropin(name):
    """The C++ reference-signature entry point `name` (e.g. "base_gauss_upper")."""
    return getattr(lib(), DROPIN_SYMBOLS[name])


def gen():
    global _gen
    if _gen is None:
        if not os.path.exists(GEN_PATH):
            raise ImportError("libsptrsv_gen.so is not built: " + GEN_PATH)
        G = ctypes.CDLL(GEN_PATH)
        _bind(G, GEN_API)
        _gen = G
    return _gen
