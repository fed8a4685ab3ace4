"""ctypes mirror of include/ncgm.h (the C ABI of the GB300 library).

The structures below follow the header field by field; they are shared by the
host-side Python API of this package and by the test suite.
"""
import ctypes as C

c_double_p = C.POINTER(C.c_double)


class Edf(C.Structure):
    """FunctionalParameters (include/EDF.hpp:20-23)."""
    _fields_ = [(n, C.c_double) for n in (
        "C0rr", "C1rr", "C0Drr", "C1Drr", "C0rt", "C1rt", "C0J2", "C1J2",
        "C0rdr", "C1rdr", "C0nJ", "C1nJ", "sigma")]


class Skyrme(C.Structure):
    """SkyrmeParameters (include/EDF.hpp:4-18)."""
    _fields_ = [(n, C.c_double) for n in (
        "W0", "W0_pr", "t0", "t1", "t2", "t3", "x0", "x1", "x2", "x3",
        "sigma", "te", "to")]


class GcgParams(C.Structure):
    """GCGParameters (include/input_parser.hpp:29-35) plus device options."""
    _fields_ = [("max_iter", C.c_int), ("tol", C.c_double),
                ("cg_steps", C.c_int), ("cg_tol", C.c_double),
                ("shift", C.c_double), ("ordering", C.c_int),
                ("precision", C.c_int), ("precond", C.c_int)]


class GcgStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int),
                ("pcg_steps_max", C.c_int), ("pcg_steps_total", C.c_int),
                ("basis_cols", C.c_int), ("max_residual", C.c_double),
                ("ms_total", C.c_double), ("ms_pcg", C.c_double),
                ("lp_columns", C.c_int)]


class Pairing(C.Structure):
    _fields_ = [("V0", C.c_double), ("window", C.c_double),
                ("basis_size", C.c_int), ("window_both", C.c_int),
                ("active", C.c_int)]


MAX_MULTIPOLE = 8  # NCGM_MAX_MULTIPOLE


class HFConfig(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("box_size", C.c_double), ("A", C.c_int),
        ("Z", C.c_int), ("edf", Edf), ("spin_orbit", C.c_int),
        ("use_j", C.c_int), ("com_corr", C.c_int), ("use_coulomb", C.c_int),
        ("density_mix", C.c_double), ("max_iterations", C.c_int),
        ("energy_tol", C.c_double), ("initial_beta", C.c_double),
        ("beta3", C.c_double), ("ws_V0", C.c_double), ("ws_r0", C.c_double),
        ("ws_diff", C.c_double), ("ws_kappa", C.c_double),
        ("wsso_V0", C.c_double), ("ws_gcg", GcgParams), ("hf_gcg", GcgParams),
        ("pairing_type", C.c_int), ("pair_n", Pairing), ("pair_p", Pairing),
        ("start_hfb_iter", C.c_int), ("pairing_threshold", C.c_double),
        ("constrain_com", C.c_int), ("curve_mode", C.c_int),
        ("mu20", C.c_double), ("constraints_tol", C.c_double),
        ("spe_tol", C.c_double), ("lp", C.c_void_p),
        ("lp_collect_every", C.c_int), ("n_multipole", C.c_int),
        ("mp_l", C.c_int * MAX_MULTIPOLE), ("mp_m", C.c_int * MAX_MULTIPOLE),
        ("mp_target", C.c_double * MAX_MULTIPOLE)]


class HFResult(C.Structure):
    _fields_ = [
        ("iterations", C.c_int), ("converged", C.c_int),
        ("E_int", C.c_double), ("E_HF", C.c_double),
        ("E_pair_n", C.c_double), ("E_pair_p", C.c_double),
        ("lambda_n", C.c_double), ("lambda_p", C.c_double),
        ("beta", C.c_double), ("gamma", C.c_double), ("wall_s", C.c_double),
        ("last_dE", C.c_double), ("t_gcg_s", C.c_double),
        ("t_fields_s", C.c_double), ("t_poisson_s", C.c_double),
        ("t_pairing_s", C.c_double), ("E_int_lagrange", C.c_double)]


ENERGY_TABLE = 16  # NCGM_ENERGY_TABLE
# labels of ncgm_hf_outputs.terms, as the reference's log prints them
ENERGY_TABLE_LABELS = (
    "E (kin)", "C0 Rho0", "C1 Rho1", "C0 nabla2Rho0", "C1 nabla2Rho1",
    "C0 tau0", "C1 tau1", "C0 div J", "C1 div J", "C0 J2", "C1 J2",
    "E coulomb direct", "E pairing neutrons", "E pairing protons",
    "E coulomb exchange", "E (REA)")


class HFOutputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "orbitals_n", "orbitals_p", "tau_n", "tau_p", "grad_rho_n",
        "grad_rho_p", "U_n", "U_p")] + [
        ("terms", C.c_double * ENERGY_TABLE),
        ("constraints_energy", C.c_double)]


NCGM_OK = 0
STATUS = {0: "NCGM_OK", 1: "NCGM_ERR_ARG", 2: "NCGM_ERR_CUDA",
          3: "NCGM_ERR_NAN", 4: "NCGM_ERR_RANK", 5: "NCGM_ERR_TIMEOUT",
          6: "NCGM_ERR_EIG", 7: "NCGM_ERR_NOMEM"}
FP64, FP32, FP32_TC = 0, 1, 2
PRECOND_JACOBI, PRECOND_LEARNED = 0, 1
NEUTRON, PROTON = 0, 1
ORDER_MATCH_PREVIOUS, ORDER_ASCENDING = 0, 1
PAIRING_NONE, PAIRING_HFB, PAIRING_BCS = 0, 1, 2

# Exported symbols and their ctypes signatures (argtypes, restype).
_vp = C.c_void_p
_i, _d = C.c_int, C.c_double
SIGNATURES = {
    "ncgm_edf_from_skyrme": ([C.POINTER(Skyrme), C.POINTER(Edf)], _i),
    "ncgm_create": ([C.POINTER(_vp), _i, _d, _i, _i], _i),
    "ncgm_destroy": ([_vp], _i),
    "ncgm_last_error": ([], C.c_char_p),
    "ncgm_sync": ([_vp], _i),
    "ncgm_set_fields": ([_vp, _i, _vp, _vp, _vp, _vp, _vp], _i),
    "ncgm_set_woods_saxon": ([_vp, _i, _i, _i, _d, _d, _d, _d, _d, _d, _d,
                              _i], _i),
    "ncgm_apply_h": ([_vp, _i, _vp, _vp, _i, _i], _i),
    "ncgm_apply_h_device": ([_vp, _i, _vp, _vp, _i, _i, _d], _i),
    "ncgm_set_stream": ([_vp, _vp], _i),
    "ncgm_gcg": ([_vp, _i, _vp, _i, _vp, _i, _i, C.POINTER(GcgParams), _vp,
                  _vp, C.POINTER(GcgStats)], _i),
    "ncgm_hf_run": ([C.POINTER(HFConfig), C.POINTER(HFResult), _vp, _vp, _vp,
                     _vp, _vp], _i),
    "ncgm_densities": ([_vp, _vp, _i, _vp, _vp, _vp, _vp], _i),
    "ncgm_lagrange_densities": ([_vp, _vp, _i, _vp, _vp, _vp, _vp], _i),
    "ncgm_hf_run_ex": ([C.POINTER(HFConfig), C.POINTER(HFResult), _vp, _vp,
                        _vp, _vp, _vp, C.POINTER(HFOutputs)], _i),
    "ncgm_shell_observables": ([_vp, _vp, _i, _vp], _i),
    "ncgm_poisson": ([_vp, _vp, _i, _vp, _vp, _vp, _vp], _i),
    "ncgm_poisson_noalloc": ([_i, _d, _vp, _i, _vp, _vp, _vp, _vp, _vp], _i),
    "ncgm_hf_run_batch": ([_vp, _i, _i, _vp, _vp, _vp, _vp], _i),
    "ncgm_gram": ([_vp, _vp, _i, _vp, _i, _vp, _i], _i),
    "ncgm_vc": ([_vp, _vp, _i, _vp, _i, _vp, _i], _i),
    "ncgm_heig": ([_vp, _vp, _i, _vp, _vp, _i], _i),
    "ncgm_lp_num_params": ([], _i),
    "ncgm_lp_create": ([C.POINTER(_vp), C.c_ulonglong], _i),
    "ncgm_lp_destroy": ([_vp], _i),
    "ncgm_lp_get_params": ([_vp, _vp], _i),
    "ncgm_lp_set_params": ([_vp, _vp], _i),
    "ncgm_lp_forward": ([_vp, _i, _i, _vp, _vp], _i),
    "ncgm_lp_gradient": ([_vp, _i, _i, _vp, _vp, _vp, _vp], _i),
    "ncgm_lp_collect": ([_vp, _vp, _i, _vp, _i, _vp, _d, _i, _d], _i),
    "ncgm_lp_dataset_size": ([_vp, _i], _i),
    "ncgm_lp_train": ([_vp, _i, _i, _d, C.c_ulonglong, _vp], _i),
    "ncgm_lp_eval": ([_vp, _i, _vp], _i),
    "ncgm_set_lp": ([_vp, _vp], _i),
    "ncgm_measure_fp64_gflops": ([_vp], _i),
    "ncgm_state_create": ([C.POINTER(_vp), C.POINTER(HFConfig)], _i),
    "ncgm_state_destroy": ([_vp], _i),
    "ncgm_state_update": ([_vp, _vp, _vp, _i, _vp, _vp, _i, _i, _i], _i),
    "ncgm_state_fields": ([_vp, _i, _vp, _vp, _vp, _vp, _vp], _i),
    "ncgm_state_densities": ([_vp, _i, _vp, _vp], _i),
    "ncgm_state_energy": ([_vp, _vp, _vp, _vp, _vp], _i),
}
UPDATE_NORMALIZE, UPDATE_TRORDER = 1, 2


def bind(lib):
    """Attach argtypes/restype to every exported symbol of `lib`."""
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib
