"""ctypes binding of libflaregb.so (the C ABI declared in include/flaregb.h).

There is no fallback: if the shared library is missing or fails to load, every
entry point raises.  Build it with ``python -m flare_gb300.build`` (or
``__graft_entry__.build()``).
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libflaregb.so")

FGB_OK, FGB_EINVAL, FGB_ENOMEM, FGB_ECUDA, FGB_ETIMEOUT, FGB_ESTALE, \
    FGB_ENOTSUP = range(7)
FGB_PREC_FP64, FGB_PREC_MIXED = 0, 1
FGB_WANT_ENERGY, FGB_WANT_FORCES, FGB_WANT_STRESS, FGB_WANT_LOCAL_VAR = \
    1, 2, 4, 8
RADIAL = {"chebyshev": 0, "weighted_chebyshev": 1, "equispaced_gaussians": 2,
          "weighted_positive_chebyshev": 3, "positive_chebyshev": 4,
          "bessel": 5, "fourier_quarter": 6, "fourier_half": 7, "fourier": 8}
CUTOFF = {"quadratic": 0, "hard": 1, "cosine": 2, "polynomial": 3, "power": 4}

# Every symbol the header declares, with (restype, argtypes).
_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_ll = ctypes.c_longlong
_pi = ctypes.POINTER(ctypes.c_int)
_pd = ctypes.POINTER(ctypes.c_double)
_pll = ctypes.POINTER(ctypes.c_longlong)
_pvp = ctypes.POINTER(ctypes.c_void_p)

SIGNATURES = {
    "fgb_last_error": (ctypes.c_char_p, []),
    "fgb_version": (_i, []),
    "fgb_profile_enable": (_i, [_i]),
    "fgb_profile_reset": (_i, []),
    "fgb_profile_n_stages": (_i, []),
    "fgb_profile_stage_name": (ctypes.c_char_p, [_i]),
    "fgb_profile_read": (_i, [_vp, _vp, _i]),
    "fgb_nlist_create": (_i, [_pvp]),
    "fgb_nlist_destroy": (_i, [_vp]),
    "fgb_nlist_build": (_i, [_vp, _i, _vp, _vp, _vp, _d, _vp]),
    "fgb_nlist_size": (_i, [_vp, _pll, _pi]),
    "fgb_nlist_export": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fgb_nlist_build_noalloc": (_i, [_vp, _vp, _i, _d, _ll, _vp, _vp, _vp,
                                     _vp, _pll, _vp]),
    "fgb_b2_create": (_i, [_pvp, _i, _i, _vp, _i, _vp, _i, _i, _i, _i, _vp]),
    "fgb_b2_destroy": (_i, [_vp]),
    "fgb_b2_size": (_i, [_vp, _pi, _pi]),
    "fgb_b2_forward": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "fgb_b2_forward_dervs": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fgb_model_create": (_i, [_pvp, _vp, _d, _d]),
    "fgb_model_destroy": (_i, [_vp]),
    "fgb_model_set": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "fgb_model_set_R_inv": (_i, [_vp, _vp]),
    "fgb_predict_sor": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "fgb_predict_dtc": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "fgb_predict": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _d, _i, _i, _vp, _vp,
                         _vp, _vp, _vp]),
    "fgb_predict_host": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _d, _i, _i, _vp,
                              _vp, _vp, _vp, _vp]),
    "fgb_envs_envs": (_i, [_vp, _vp, _i, _vp, _vp, _i, _i, _d, _d, _vp,
                           _vp]),
    "fgb_envs_struc": (_i, [_vp, _d, _d, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fgb_self_kernel_struc": (_i, [_vp, _d, _d, _vp, _vp, _vp, _vp]),
    "fgb_struc_struc": (_i, [_vp, _d, _d, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fgb_predict_plain": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "fgb_oz_dgemm_nt": (_i, [_i, _i, _i, _vp, _ll, _vp, _ll, _vp, _ll, _vp]),
    "fgb_oz_dgemm_nt_slices": (_i, [_i, _i, _i, _i, _vp, _ll, _vp, _ll, _vp,
                                    _ll, _vp]),
    "fgb_oz_sgemm_nt": (_i, [_i, _i, _i, _vp, _ll, _vp, _ll, _vp, _ll, _vp]),
    "fgb_md_create": (_i, [_vp, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _d, _i]),
    "fgb_md_destroy": (_i, [_vp]),
    "fgb_md_set_model": (_i, [_vp, _vp]),
    "fgb_md_step": (_i, [_vp, _i, _d, _d, _vp]),
    "fgb_md_set_graphs": (_i, [_vp, _i, _d]),
    "fgb_md_stats": (_i, [_vp, _vp]),
    "fgb_model_mapping": (_i, [_vp, _vp, _vp]),
    "fgb_model_fold_guard": (_i, [_vp, _vp, _vp, _vp]),
    "fgb_model_mixed_plan": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "fgb_model_slice_plan": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "fgb_model_set_slices": (_i, [_vp, _i, _i]),
    "fgb_wait_expiry_check": (_i, [ctypes.c_longlong, _vp, _vp]),
    "fgb_qr_thin_q": (_i, [_i, _i, _vp, _vp, _vp]),
    "fgb_mapped_create": (_i, [_pvp, _vp, _i, _i, _vp, _vp]),
    "fgb_mapped_destroy": (_i, [_vp]),
    "fgb_mapped_predict": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _d, _i, _vp,
                                _vp, _vp, _vp, _vp, _i, _vp]),
    "fgb_tune_set_mode": (_i, [_i]),
    "fgb_tune_force": (_i, [_i, _i]),
    "fgb_tune_clear": (_i, []),
    "fgb_tune_count": (_i, []),
    "fgb_tune_entry": (_i, [_i, _vp, _vp]),
    "fgb_md_read": (_i, [_vp] + [_vp] * 8 + [_vp]),
    "fgb_serve_start": (_i, [_pvp, _vp, _i, _ll, _i, _d, _i, _i]),
    "fgb_serve_submit": (_i, [_vp, _i, _vp, _vp, _vp, _pll]),
    "fgb_serve_poll": (_i, [_vp, _ll, _pi, _vp, _vp, _vp, _vp, _pd]),
    "fgb_serve_stats": (_i, [_vp, _pll, _pll, _pll]),
    "fgb_serve_stop": (_i, [_vp]),
    "fgb_solve_qr": (_i, [_i, _i, _vp, _vp, _vp, _vp, _d, _vp, _vp, _vp,
                          _vp]),
    "fgb_cholesky": (_i, [_i, _vp, _vp]),
    "fgb_trtri_lower": (_i, [_i, _vp, _vp, _vp]),
    "fgb_solve_products": (_i, [_i, _vp, _vp, _vp, _vp, _vp]),
}

_lib = None


def lib():
    """Load libflaregb.so once; raise if it is absent (no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libflaregb.so is not built (expected at %s); run "
                "`python -m flare_gb300.build`" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class FlareGBError(RuntimeError):
    pass


def check(rc, what=""):
    """Map an fgb status to the exception the reference raises."""
    if rc == FGB_OK:
        return
    msg = lib().fgb_last_error().decode(errors="replace")
    if what:
        msg = f"{what}: {msg}"
    if rc == FGB_EINVAL:
        raise ValueError(msg)
    if rc == FGB_ENOMEM:
        raise MemoryError(msg)
    if rc == FGB_ENOTSUP:
        raise NotImplementedError(msg)
    if rc == FGB_ESTALE:
        raise RuntimeError(msg)
    raise FlareGBError(f"status {rc}: {msg}")


def ptr(t):
    """Raw pointer of a torch tensor or numpy array (None -> NULL)."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return ctypes.c_void_p(t.data_ptr())
    return ctypes.c_void_p(t.ctypes.data)


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)
