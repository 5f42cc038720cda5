"""ctypes declarations of include/fjgpu.h (the C ABI of libfjgpu.so)."""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfjgpu.so")

DP = C.POINTER(C.c_double)

FJ_OK = 0
FJ_DF_DPL, FJ_DF_QUASIISO = 0, 1
FJ_PREC_FP64, FJ_PREC_MIXED = 0, 1
FJ_TWOCOMP_SUMMED, FJ_TWOCOMP_REFERENCE = 0, 1
FJ_JQUAD_QAGS = 0
FJ_POISSON_QAGS, FJ_POISSON_CUMULATIVE = 0, 1
FJ_GUESS = {"Hernquist": 0, "Isochrone": 1, "NFW": 2, "NFWext": 3}


class fj_potential(C.Structure):
    _fields_ = [("nr", C.c_int), ("npoly", C.c_int), ("ar", C.c_void_p), ("phil", C.c_void_p),
                ("Pr", C.c_void_p), ("Pr2", C.c_void_p)]


class fj_delta_table(C.Structure):
    _fields_ = [("ngrid", C.c_int), ("Egrid", C.c_void_p), ("Dgrid", C.c_void_p)]


class fj_df_params(C.Structure):
    _fields_ = [("kind", C.c_int)] + [(n, C.c_double) for n in
                                      ("alpha", "beta", "J0", "mass", "dphi_h", "dz_h", "dphi_g", "dz_g", "chi", "k")]


class fj_quad_rule(C.Structure):
    _fields_ = [("nq", C.c_int), ("xq", DP), ("wq", DP), ("jquad", C.c_int), ("precision", C.c_int)]


class fj_moment_stats(C.Structure):
    _fields_ = [("nodes", C.c_longlong), ("bound", C.c_longlong), ("failures", C.c_longlong),
                ("kernel_ms", C.c_double), ("escalated", C.c_longlong), ("fail_quad", C.c_longlong),
                ("fail_bracket", C.c_longlong), ("fail_root", C.c_longlong), ("resolved64", C.c_longlong)]


class fj_batch_item(C.Structure):
    _fields_ = [("pot", fj_potential), ("delta", fj_delta_table), ("df", fj_df_params), ("ngauss", C.c_int),
                ("grids6", C.c_void_p)]


class fj_surrogate_schedule(C.Structure):
    _fields_ = [("exact_first", C.c_int), ("exact_last", C.c_int), ("samples", C.c_longlong),
                ("epochs_first", C.c_int), ("epochs", C.c_int), ("lr", C.c_float), ("seed", C.c_ulonglong),
                ("r_exact", C.c_double), ("audit_stride", C.c_int), ("audit_tol", C.c_double)]


class fj_surrogate_report(C.Structure):
    _fields_ = [("surrogate_iterations", C.c_int), ("fallback_iterations", C.c_int), ("fits", C.c_int),
                ("last_audit_err", C.c_double), ("max_audit_err", C.c_double), ("last_fit_loss", C.c_double),
                ("surrogate_ms", C.c_double), ("exact_ms", C.c_double), ("fit_ms", C.c_double)]


class fj_model_config(C.Structure):
    _fields_ = [("nr", C.c_int), ("ngauss", C.c_int), ("npoly", C.c_int), ("ngrid", C.c_int),
                ("rmin", C.c_double), ("rmax", C.c_double), ("guess", C.c_int),
                ("mass", C.c_double), ("r0", C.c_double), ("q", C.c_double),
                ("df", fj_df_params), ("rule", fj_quad_rule), ("itermax", C.c_int), ("tol", C.c_double),
                ("Egrid_in", DP), ("Dgrid_in", DP), ("ncomp", C.c_int), ("guess2", C.c_int),
                ("mass2", C.c_double), ("r0_2", C.c_double), ("q2", C.c_double), ("df2", fj_df_params),
                ("twocomp_order", C.c_int), ("ar_in", DP), ("phil_in", DP), ("Pr_in", DP), ("Pr2_in", DP),
                ("delta_gpu", C.c_int), ("delta_every", C.c_int), ("ext_phil", DP), ("ext_Pr", DP), ("ext_Pr2", DP),
                ("accel", C.c_int), ("accel_beta", C.c_double)]


class fj_model_result(C.Structure):
    _fields_ = [(n, DP) for n in ("ar", "coef6", "phil", "Pr", "Pr2", "Egrid", "Dgrid", "grids6")] + [
        ("vir7", C.c_double * 7), ("iterations", C.c_int), ("last_change", C.c_double),
        ("bound", C.c_longlong), ("failures", C.c_longlong), ("wall_ms", C.c_double), ("kernel_ms", C.c_double),
        ("setup_ms", C.c_double), ("coef6_2", DP), ("vir7_2", C.c_double * 7)]


P = C.POINTER
FJ_ANDERSON_MAX_DEPTH = 8
FJ_LOS_SIGMA, FJ_LOS_LINE, FJ_LOS_PVPHI, FJ_LOS_PVZ, FJ_LOS_PVR = range(5)
CTX = C.c_void_p
SIGNATURES = {
    "fj_version": ([], C.c_char_p),
    "fj_ctx_create": ([C.c_int, P(C.c_void_p)], C.c_int),
    "fj_anderson_reset": ([CTX, C.c_int, C.c_double], C.c_int),
    "fj_anderson_step": ([CTX, C.c_int, C.c_int, C.c_void_p, C.c_void_p, DP], C.c_int),
    "fj_anderson_create": ([C.c_int, C.c_double, P(C.c_void_p)], C.c_int),
    "fj_anderson_destroy": ([C.c_void_p], C.c_int),
    "fj_anderson_host_step": ([C.c_void_p, C.c_int, C.c_int, DP, DP, DP], C.c_int),
    "fj_ctx_destroy": ([CTX], C.c_int),
    "fj_ctx_set_stream": ([CTX, C.c_void_p], C.c_int),
    "fj_ctx_own_stream": ([CTX], C.c_void_p),
    "fj_ctx_synchronize": ([CTX], C.c_int),
    "fj_last_error": ([CTX], C.c_char_p),
    "fj_moments": ([CTX, P(fj_potential), P(fj_delta_table), P(fj_df_params), P(fj_quad_rule), C.c_int,
                    C.c_void_p, P(fj_moment_stats)], C.c_int),
    "fj_moments_points": ([CTX, P(fj_potential), P(fj_delta_table), P(fj_df_params), P(fj_quad_rule),
                           C.c_void_p, C.c_int, C.c_void_p, P(fj_moment_stats)], C.c_int),
    "fj_moments_batch": ([CTX, C.c_int, P(fj_batch_item), P(fj_quad_rule), P(fj_moment_stats)], C.c_int),
    "fj_run_model_batch": ([CTX, C.c_int, P(fj_model_config), P(fj_model_result), C.c_int], C.c_int),
    "fj_tc_gemm": ([C.c_int] * 3 + [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                     C.c_void_p], C.c_int),
    "fj_surrogate_create": ([CTX, C.c_int, C.c_ulonglong, P(C.c_void_p)], C.c_int),
    "fj_surrogate_destroy": ([C.c_void_p], C.c_int),
    "fj_surrogate_nparam": ([C.c_void_p], C.c_longlong),
    "fj_surrogate_params": ([C.c_void_p, DP, DP], C.c_int),
    "fj_surrogate_gradients": ([C.c_void_p, C.c_void_p, C.c_void_p, DP, DP], C.c_int),
    "fj_surrogate_train": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_float, DP], C.c_int),
    "fj_surrogate_predict": ([C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p], C.c_int),
    "fj_set_action_output": ([CTX, C.c_void_p], C.c_int),
    "fj_surrogate_fit": ([C.c_void_p, P(fj_potential), P(fj_df_params), C.c_int, P(fj_quad_rule), C.c_void_p,
                          C.c_void_p, C.c_longlong, C.c_ulonglong, C.c_int, C.c_float, DP], C.c_int),
    "fj_surrogate_moments": ([C.c_void_p, P(fj_potential), P(fj_df_params), P(fj_quad_rule), C.c_int, C.c_void_p,
                              DP, C.c_int], C.c_int),
    "fj_run_model_surrogate": ([CTX, P(fj_model_config), P(fj_surrogate_schedule), C.c_void_p, P(fj_model_result),
                                P(fj_surrogate_report)], C.c_int),
    "fj_set_mixed_config": ([CTX, C.c_int, C.c_int], C.c_int),
    "fj_get_mixed_config": ([CTX, P(C.c_int), P(C.c_int)], C.c_int),
    "fj_autotune_mixed": ([CTX, P(fj_potential), P(fj_delta_table), P(fj_df_params), P(fj_quad_rule), C.c_void_p,
                           C.c_int, C.c_void_p, DP, DP], C.c_int),
    "fj_legendre_project": ([CTX, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "fj_poisson": ([CTX, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "fj_poisson_noalloc": ([C.c_int, C.c_int] + [C.c_void_p] * 6, C.c_int),
    "fj_set_poisson": ([CTX, C.c_int], C.c_int),
    "fj_get_poisson": ([CTX, P(C.c_int)], C.c_int),
    "fj_poisson_noalloc_stack": ([P(C.c_size_t), P(C.c_size_t)], C.c_int),
    "fj_sum_potentials": ([CTX, C.c_int] + [C.c_void_p] * 9, C.c_int),
    "fj_compute_new_phi": ([CTX, P(fj_potential), P(fj_delta_table), P(fj_df_params), P(fj_quad_rule), C.c_int,
                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, P(fj_moment_stats)], C.c_int),
    "fj_actions": ([CTX, P(fj_potential), P(fj_delta_table), C.c_void_p, C.c_size_t, C.c_int, C.c_void_p], C.c_int),
    "fj_potential_eval": ([CTX, P(fj_potential), C.c_void_p, C.c_size_t, C.c_void_p], C.c_int),
    "fj_los": ([CTX, P(fj_potential), P(fj_delta_table), P(fj_df_params), P(fj_quad_rule), C.c_void_p, C.c_int,
                C.c_void_p, C.c_int, C.c_void_p, P(fj_moment_stats)], C.c_int),
    "fj_tanh_sinh01": ([DP, DP], C.c_int),
    "fj_tabulate_delta_batch": ([CTX, C.c_int, P(fj_potential), C.c_int, C.c_void_p, C.c_void_p, P(C.c_int)],
                                C.c_int),
    "fj_vir2": ([CTX, P(fj_potential), C.c_int, C.c_void_p, DP], C.c_int),
    "fj_measure_fma_peak": ([C.c_int, DP], C.c_int),
    "fj_log_grid": ([C.c_double, C.c_double, C.c_int, DP], C.c_int),
    "fj_gauleg": ([C.c_double, C.c_double, C.c_int, DP, DP], C.c_int),
    "fj_guess_rhl": ([C.c_int, C.c_int, C.c_int, DP, C.c_int, C.c_double, C.c_double, C.c_double, DP], C.c_int),
    "fj_tabulate_delta": ([P(fj_potential), C.c_int, DP, DP], C.c_int),
    "fj_write_out": ([C.c_char_p, C.c_int, C.c_int, C.c_int, DP, DP, DP], C.c_int),
    "fj_write_out_digits": ([C.c_char_p, C.c_int, C.c_int, C.c_int, DP, DP, DP, C.c_int], C.c_int),
    "fj_read_out": ([C.c_char_p, P(C.c_int), P(C.c_int), P(C.c_int), DP, DP, DP], C.c_int),
    "fj_run_model": ([CTX, P(fj_model_config), P(fj_model_result)], C.c_int),
}

_lib = None


def load(build_if_missing=True):
    """Load libfjgpu.so (building it first when a source is newer).  Raises if it cannot."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        from . import build as _b
        _b.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libfjgpu.so is missing at {LIB_PATH}; run python -m fjmodels_gb300.build")
    lib = C.CDLL(LIB_PATH)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib
