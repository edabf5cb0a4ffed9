"""ctypes binding of the C ABI declared in include/libkriging_gb300.h.

The shared library is built in-tree (libkriging_gb300/_build/liblkgpu.so).  There is no CPU fallback: if the library
is missing or a call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
SO = PKG / "_build" / "liblkgpu.so"
HEADER = PKG.parent / "include" / "libkriging_gb300.h"

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_cp = ctypes.c_char_p
_i = ctypes.c_int
_d = ctypes.c_double

# name -> (restype, argtypes)
_SIGS = {
    "lkg_get_last_error": (_cp, []),
    "lkg_kriging_new": (_vp, [_cp, _cp]),
    "lkg_kriging_new_fit": (_vp, [_dp, _i, _dp, _i, _dp, _i, _i, _cp, _cp, _cp, _i, _cp, _cp, _dp, _i, _dp, _i, _i,
                                  _dp, _i, _i, _dp, _i]),
    "lkg_kriging_delete": (None, [_vp]),
    "lkg_kriging_fit": (_i, [_vp, _dp, _i, _dp, _i, _dp, _i, _i, _cp, _i, _cp, _cp]),
    "lkg_kriging_fit_params": (_i, [_vp, _dp, _i, _dp, _i, _i, _cp, _i, _cp, _cp, _dp, _i, _dp, _i, _i, _dp, _i, _i,
                                    _dp, _i]),
    "lkg_kriging_predict": (_i, [_vp, _dp, _i, _i, _i, _i, _i, _dp, _dp, _dp, _dp, _dp]),
    "lkg_kriging_summary": (_cp, [_vp]),
    "lkg_kriging_copy": (_vp, [_vp]),
    "lkg_kriging_update": (_i, [_vp, _dp, _i, _dp, _i, _dp, _i, _i, _i]),
    "lkg_kriging_save": (_i, [_vp, _cp]),
    "lkg_kriging_load": (_vp, [_cp]),
    "lkg_kriging_cov_mat": (_i, [_vp, _dp, _i, _i, _dp, _i, _i, _dp]),
    "lkg_kriging_get_F": (_i, [_vp, _dp, _ip, _ip]),
    "lkg_oz7_mode_check": (_i, [_i, _i, _i, _i, _dp, _dp, _i, _dp, _ip]),
    "lkg_kriging_log_likelihood_fun": (_i, [_vp, _dp, _i, _i, _i, _dp, _dp, _dp]),
    "lkg_kriging_log_likelihood": (_d, [_vp]),
    "lkg_kriging_leave_one_out_fun": (_i, [_vp, _dp, _i, _i, _dp, _dp]),
    "lkg_kriging_leave_one_out": (_d, [_vp]),
    "lkg_kriging_leave_one_out_vec": (_i, [_vp, _dp, _i, _dp, _dp]),
    "lkg_kriging_log_marg_post_fun": (_i, [_vp, _dp, _i, _i, _dp, _dp]),
    "lkg_kriging_log_marg_post": (_d, [_vp]),
    "lkg_kriging_log_likelihood_fun_batch": (_i, [_vp, _dp, _i, _i, _i, _dp, _dp]),
    "lkg_kriging_log_likelihood_fun_bench": (_i, [_vp, _dp, _i, _i, _dp, _dp, ctypes.c_char_p, _i]),
    "lkg_kriging_log_likelihood_fun_batch_bench": (_i, [_vp, _dp, _i, _i, _i, _dp, _dp, ctypes.c_char_p, _i]),
    "lkg_kriging_kernel": (_cp, [_vp]),
    "lkg_kriging_optim": (_cp, [_vp]),
    "lkg_kriging_objective": (_cp, [_vp]),
    "lkg_kriging_is_normalize": (_i, [_vp]),
    "lkg_kriging_regmodel": (_cp, [_vp]),
    "lkg_kriging_get_X": (_i, [_vp, _dp, _ip, _ip]),
    "lkg_kriging_get_centerX": (_i, [_vp, _dp, _ip]),
    "lkg_kriging_get_scaleX": (_i, [_vp, _dp, _ip]),
    "lkg_kriging_get_y": (_i, [_vp, _dp, _ip]),
    "lkg_kriging_get_centerY": (_d, [_vp]),
    "lkg_kriging_get_scaleY": (_d, [_vp]),
    "lkg_kriging_get_T": (_i, [_vp, _dp, _ip, _ip]),
    "lkg_kriging_get_M": (_i, [_vp, _dp, _ip, _ip]),
    "lkg_kriging_get_z": (_i, [_vp, _dp, _ip]),
    "lkg_kriging_get_beta": (_i, [_vp, _dp, _ip]),
    "lkg_kriging_is_beta_estim": (_i, [_vp]),
    "lkg_kriging_get_theta": (_i, [_vp, _dp, _ip]),
    "lkg_kriging_is_theta_estim": (_i, [_vp]),
    "lkg_kriging_get_sigma2": (_d, [_vp]),
    "lkg_kriging_is_sigma2_estim": (_i, [_vp]),
    "lkg_kriging_noise_model": (_cp, [_vp]),
    "lkg_kriging_get_nugget": (_d, [_vp]),
    "lkg_kriging_is_nugget_estim": (_i, [_vp]),
    "lkg_set_num_nugget": (None, [_d]),
    "lkg_get_num_nugget": (_d, []),
    "lkg_check_chol_rcond": (None, [_i]),
    "lkg_set_chol_warning": (None, [_i]),
    "lkg_optim_use_reparametrize": (None, [_i]),
    "lkg_optim_set_theta_lower_factor": (None, [_d]),
    "lkg_optim_set_theta_upper_factor": (None, [_d]),
    "lkg_optim_use_variogram_bounds_heuristic": (None, [_i]),
    "lkg_optim_set_log_level": (None, [_i]),
    "lkg_optim_set_max_iteration": (None, [_i]),
    "lkg_optim_set_gradient_tolerance": (None, [_d]),
    "lkg_optim_set_objective_rel_tolerance": (None, [_d]),
    "lkg_optim_set_max_restart": (None, [_i]),
    "lkg_device_name": (_cp, []),
    "lkg_probe_fp64_peak": (_i, [_dp]),
    "lkg_probe_dmma_peak": (_i, [_dp]),
    "lkg_stats_enable": (None, [_i]),
    "lkg_stats_reset": (None, []),
    "lkg_stats_report": (_i, [ctypes.c_char_p, _i]),
    "lkg_kriging_set_precision": (_i, [_vp, _i]),
    "lkg_kriging_get_precision": (_i, [_vp]),
    "lkg_kriging_last_slices": (_i, [_vp]),
    "lkg_kriging_eval_counts": (_i, [_vp, _vp, _vp]),
    "lkg_kriging_autotune_precision": (_i, [_vp, _dp, _i, _d, _d]),
    "lkg_kriging_autotune_lookahead": (_i, [_vp, _dp, _i]),
    "lkg_autotune_enable": (None, [_i]),
    "lkg_autotune_record": (_i, [_cp, _ip, _dp, _i]),
    "lkg_autotune_lookup": (_i, [_cp, _i]),
    "lkg_autotune_report": (_i, [ctypes.c_char_p, _i]),
    "lkg_autotune_save": (_i, [_cp]),
    "lkg_autotune_load": (_i, [_cp]),
    "lkg_autotune_clear": (None, []),
    "lkg_ozaki_gemm_check": (_i, [_i, _i, _i, _dp, _dp, _i, _dp]),
    "lkg_kriging_log_likelihood_vecchia_fun": (_i, [_vp, _dp, _i, _i, _dp, _dp]),
    "lkg_kriging_set_vecchia_exact_commit": (_i, [_vp, _i]),
    "lkg_kriging_vecchia_neighbors": (_i, [_vp]),
    "lkg_kriging_is_vecchia_light": (_i, [_vp]),
    "lkg_kriging_get_vecchia_sets": (_i, [_vp, _ip, _ip, _ip, _ip]),
    "lkg_vecchia_sets": (_i, [_i, _i, _dp, _i, _ip, _ip]),
    "lkg_kriging_predict_vecchia": (_i, [_vp, _dp, _i, _i, _i, _i, _dp, _dp]),
    "lkg_set_tensor_path": (_i, [_i]),
    "lkg_get_tensor_path": (_i, []),
    "lkg_set_digit_tile": (_i, [_i]),
    "lkg_get_digit_tile": (_i, []),
    "lkg_set_lookahead": (_i, [_i]),
    "lkg_get_lookahead": (_i, []),
    "lkg_set_graphs": (_i, [_i]),
    "lkg_vecchia_sets_noalloc": (_i, [_i, _i, _vp, _i, _vp, _vp, _vp]),
    "lkg_vecchia_shard_new": (_vp, [_cp, _i, _i, _i, _dp, _dp, _dp, _ip, _ip, _i, _i, _i]),
    "lkg_vecchia_shard_delete": (None, [_vp]),
    "lkg_vecchia_shard_sums1": (_i, [_vp, _dp, _i, _dp, _vp, _ip]),
    "lkg_vecchia_shard_sums2": (_i, [_vp, _dp, _i, _dp]),
    "lkg_vecchia_gls_beta": (_i, [_i, _dp, _dp]),
    "lkg_vecchia_finish": (_i, [_i, _i, ctypes.c_double, _dp, _i, _dp, _dp, _dp]),
    "lkg_nested_kriging_new_fit": (_vp, [_dp, _i, _dp, _i, _i, _cp, _i, _cp, _cp, _i, _vp, _i, _cp, _cp, _cp, _dp, _i,
                                         _dp, _i, _i, _dp, _i, _i]),
    "lkg_nested_kriging_delete": (None, [_vp]),
    "lkg_nested_kriging_fit": (_i, [_vp, _dp, _i, _dp, _i, _i, _i, _vp, _i, _cp, _cp, _cp, _dp, _i, _dp, _i, _i, _dp,
                                    _i, _i]),
    "lkg_nested_kriging_predict": (_i, [_vp, _dp, _i, _i, _i, _dp, _dp]),
    "lkg_nested_kriging_summary": (_cp, [_vp]),
    "lkg_nested_kriging_kernel": (_cp, [_vp]),
    "lkg_nested_kriging_aggregation": (_cp, [_vp]),
    "lkg_nested_kriging_nb_groups": (_i, [_vp]),
    "lkg_nested_kriging_get_theta": (_i, [_vp, _dp, _ip]),
    "lkg_nested_kriging_get_sigma2": (_d, [_vp]),
    "lkg_nested_kriging_get_beta0": (_d, [_vp]),
    "lkg_nested_kriging_new": (_vp, [_cp, _cp, _cp, _i]),
    "lkg_nested_kriging_fit_groups": (_i, [_vp, _dp, _i, _dp, _i, _i, _ip, _i, _cp, _cp, _cp, _dp, _i, _dp, _i, _i,
                                           _dp, _i, _i]),
    "lkg_nested_kriging_get_groups": (_i, [_vp, _ip, _ip]),
    "lkg_nested_kriging_submodel": (_vp, [_vp, _i]),
    "lkg_nested_kriging_set_precision": (_i, [_vp, _i]),
    "lkg_nested_kriging_set_predict_chunk": (_i, [_vp, _i]),
    "lkg_nested_kriging_log_likelihood_groups": (_i, [_vp, _dp, _i, _i, _i, _dp, _dp]),
    "lkg_nested_kriging_get_group_estimates": (_i, [_vp, _dp, _dp, _dp, _ip, _ip]),
}

_lib = None


class LibKrigingError(RuntimeError):
    pass


def header_symbols():
    """Function names declared in include/libkriging_gb300.h."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lkg_[A-Za-z0-9_]+)\s*\(", text)))


def load():
    """Load the in-tree shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not SO.exists():
        raise LibKrigingError("GPU library %s is missing: run `python -c 'import __graft_entry__ as g; g.build()'` "
                              "(there is no CPU fallback)" % SO)
    lib = ctypes.CDLL(str(SO))
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    return load().lkg_get_last_error().decode()


def check(rc):
    if rc != 0:
        raise LibKrigingError(last_error())
    return rc


def ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def f64(a):
    """float64, column-major (Fortran) contiguous copy or view."""
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def cstr(s):
    return None if s is None else s.encode()
