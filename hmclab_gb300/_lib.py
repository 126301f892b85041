"""ctypes binding of the C ABI declared in include/hmclab_gb300.h.

The shared library is built in-tree (`hmclab_gb300/libhmclab_gb300.so`, see
`build.py`).  There is no CPU fallback: every device operation raises
`DeviceUnavailableError` when the library or a CUDA device is missing.
"""
import ctypes as _ct
import os as _os
import threading as _threading

from hmclab_gb300.Helpers.CustomExceptions import DeviceUnavailableError, DeviceTimeoutError

_HERE = _os.path.dirname(_os.path.abspath(__file__))
LIB_PATH = _os.path.join(_HERE, "libhmclab_gb300.so")

HMC_OK = 0
HMC_ERR_INVALID_ARG = 1
HMC_ERR_CUDA = 2
HMC_ERR_TIMEOUT = 3
HMC_ERR_NONFINITE = 4
HMC_ERR_UNSUPPORTED = 5

HMC_F32 = 0
HMC_F64 = 1

HMC_MASS_UNIT = 0
HMC_MASS_DIAG = 1
HMC_MASS_FULL = 2

HMC_FLAG_OUT_OF_BOUNDS = 1

HMC_CSR_GATHER, HMC_CSR_GATHER4, HMC_CSR_SLAB = 0, 1, 2

c_void_p = _ct.c_void_p
c_int = _ct.c_int
c_int32 = _ct.c_int32
c_int64 = _ct.c_int64
c_uint32 = _ct.c_uint32
c_uint64 = _ct.c_uint64
c_double = _ct.c_double
c_char_p = _ct.c_char_p


class HmcChains(_ct.Structure):
    """Mirror of `hmc_chains` in include/hmclab_gb300.h (field order matters)."""

    _fields_ = [
        ("dtype", c_int32),
        ("mass_kind", c_int32),
        ("dims", c_int64),
        ("chains", c_int64),
        ("q_cur", c_void_p),
        ("q", c_void_p),
        ("p", c_void_p),
        ("g", c_void_p),
        ("v", c_void_p),
        ("mass_diag", c_void_p),
        ("mass_inv_diag", c_void_p),
        ("mass_chol", c_void_p),
        ("mass_inv", c_void_p),
        ("lower", c_void_p),
        ("upper", c_void_p),
        ("eps", c_void_p),
        ("eps_local", c_void_p),
        ("x_cur", c_void_p),
        ("x_prop", c_void_p),
        ("k_cur", c_void_p),
        ("k_prop", c_void_p),
        ("accepted", c_void_p),
        ("flags", c_void_p),
        ("proposal", c_void_p),
        ("seed", c_uint64),
        ("randomize_stepsize", c_int32),
        ("autotune", c_int32),
        ("target_acceptance", c_double),
        ("learning_rate", c_double),
        ("minimal_stepsize", c_double),
        ("stream_z", c_void_p),
        ("stream_eps", c_void_p),
        ("stream_u", c_void_p),
        ("stream_len", c_int64),
        ("ring_q", c_void_p),
        ("ring_x", c_void_p),
        ("ring_slots", c_int64),
        ("thinning", c_int64),
        ("rec_stepsize", c_void_p),
        ("rec_acceptance", c_void_p),
        ("rec_len", c_int64),
        ("beta", c_void_p),
    ]


class HmcFwi(_ct.Structure):
    """Mirror of `hmc_fwi` in include/hmclab_gb300.h."""

    _fields_ = [
        ("nx", c_int32),
        ("nz", c_int32),
        ("nt", c_int32),
        ("nrec", c_int32),
        ("chains", c_int64),
        ("h", _ct.c_float),
        ("dt", _ct.c_float),
        ("w", _ct.c_float),
    ] + [(n, c_void_p) for n in (
        "taper", "stf_host", "rec_map", "rho", "vp", "vs", "bx", "bz", "l2m", "lam", "muxz", "vx", "vz", "sxx",
        "szz", "sxz", "store", "rec", "obs", "resid", "avx", "avz", "asxx", "aszz", "asxz", "g_bx", "g_bz",
        "g_l2m", "g_lam", "g_muxz", "t1", "t2", "t3", "t4", "t5", "partial", "status")] + [
        ("snapshot_interval", c_int32)]


class HmcFwiSource(_ct.Structure):
    """Mirror of `hmc_fwi_source` in include/hmclab_gb300.h."""

    _fields_ = [
        ("x", c_int32),
        ("z", c_int32),
        ("mxx", _ct.c_float),
        ("mzz", _ct.c_float),
        ("mxz", _ct.c_float),
        ("stf_host", c_void_p),
    ]


HMC_SCHEDULE_MAX = 64


class HmcSchedule(_ct.Structure):
    """Mirror of `hmc_schedule` in include/hmclab_gb300.h."""

    _fields_ = [
        ("first_drift", _ct.c_double),
        ("steps", c_int32),
        ("gradient", c_int32 * HMC_SCHEDULE_MAX),
        ("kick", _ct.c_double * HMC_SCHEDULE_MAX),
        ("drift", _ct.c_double * HMC_SCHEDULE_MAX),
    ]


class HmcCsrSlabs(_ct.Structure):
    """Mirror of `hmc_csr_slabs` in include/hmclab_gb300.h."""

    _fields_ = [
        ("col", c_void_p),
        ("val", c_void_p),
        ("slab_ptr", c_void_p),
        ("rows", c_int64),
        ("cols", c_int64),
        ("slab", c_int32),
        ("rows_per_warp", c_int32),
        ("row_ptr", c_void_p),
        ("kernel", c_int32),
        ("reserved", c_int32),
    ]


class HmcDenseGroup(_ct.Structure):
    """Mirror of `hmc_dense_group` in include/hmclab_gb300.h."""

    _fields_ = [
        ("chains", c_void_p),
        ("GtG", c_void_p),
        ("Gtd0", c_void_p),
        ("dtd", _ct.c_double),
        ("prior", _ct.c_int),
        ("prior_mean", c_void_p),
        ("prior_w", c_void_p),
    ]


class HmcMlpOut(_ct.Structure):
    """Mirror of `hmc_mlp_out` in include/hmclab_gb300.h."""

    _fields_ = [
        ("z", c_void_p),
        ("ldz", c_int64),
        ("act", c_void_p),
        ("ld_act", c_int64),
        ("act_t", c_void_p),
        ("ld_act_t", c_int64),
        ("y", c_void_p),
        ("ldy", c_int64),
        ("g_state", c_void_p),
        ("out_scale", c_void_p),
        ("out_shift", c_void_p),
        ("g", c_void_p),
        ("accumulate", c_int32),
    ]


HMC_MLP_HIDDEN, HMC_MLP_OUT, HMC_MLP_BACK, HMC_MLP_WGRAD = 0, 1, 2, 3
HMC_POT_DELTA2, HMC_POT_DELTA1, HMC_POT_DBAR1, HMC_POT_DBAR2, HMC_POT_ZBAR1 = 0, 1, 2, 3, 4

P = c_void_p
I = c_int
I64 = c_int64
D = c_double
S = c_void_p  # stream

# name -> argtypes (restype is int unless listed in _RESTYPES)
SIGNATURES = {
    "hmc_version": [],
    "hmc_last_error": [],
    "hmc_launch_count": [],
    "hmc_set_wait_limits": [c_uint64, I],
    "hmc_stream_capturing": [S, P],
    "hmc_csr_slab_misfit": [P, I64, P, P, P, P, P, P, I, S],
    "hmc_csr_slab_gradient": [P, P, I64, P, P, P, P, P, P, I, S],
    "hmc_philox_normal": [I, I64, I64, c_uint64, c_uint64, c_uint32, P, S],
    "hmc_philox_raw": [I64, c_uint32, c_uint32, c_uint32, c_uint32, c_uint32, c_uint32, P, S],
    "hmc_begin_trajectory": [P, D, S],
    "hmc_kick_drift": [P, D, D, S],
    "hmc_end_trajectory": [P, S],
    "hmc_kinetic_energy": [P, P, P, S],
    "hmc_kinetic_energy_gradient": [P, P, P, S],
    "hmc_normal_diag_misfit": [I, I64, I64, P, P, P, P, I, S],
    "hmc_normal_diag_gradient": [I, I64, I64, P, P, P, P, I, S],
    "hmc_normal_full_misfit": [I, I64, I64, P, P, P, P, P, I, S],
    "hmc_normal_full_gradient": [I, I64, I64, P, P, P, P, P, I, S],
    "hmc_laplace_misfit": [I, I64, I64, P, P, P, P, I, S],
    "hmc_laplace_gradient": [I, I64, I64, P, P, P, P, I, S],
    "hmc_dense_premul_gradient": [I, I64, I64, P, P, P, P, I, S],
    "hmc_dense_premul_misfit": [I, I64, I64, P, P, P, D, P, P, I, S],
    "hmc_dense_resid_misfit": [I, I64, I64, I64, P, P, P, P, P, P, I, S],
    "hmc_dense_resid_gradient": [I, I64, I64, I64, P, P, P, P, P, P, P, I, S],
    "hmc_dense_resid_misfit_noalloc": [I, I64, I64, I64, P, P, P, P, P, I, S],
    "hmc_csr_misfit": [I, I64, I64, I64, P, P, P, P, P, P, P, P, I, S],
    "hmc_csr_gradient": [I, I64, I64, I64, P, P, P, P, P, P, P, P, P, P, P, I, S],
    "hmc_srcloc3d_misfit": [I, I64, I64, I64, P, P, P, P, P, P, I, D, P, I, S],
    "hmc_srcloc3d_gradient": [I, I64, I64, I64, P, P, P, P, P, P, I, D, P, I, S],
    "hmc_gemm": [I, I64, I64, I64, D, P, P, P, P, I, S],
    "hmc_exchange": [P, I64, P, P, P, P, S],
    "hmc_persistent_dense": [P, P, P, D, I, P, P, P, I64, I, I, S],
    "hmc_persistent_dense_groups": [P, I, P, I64, I, I, S],
    "hmc_gemm_splitk": [I, I64, I64, I64, D, P, P, P, I, P, I64, S],
    "hmc_split_bf16": [I64, I64, P, I64, P, P, S],
    "hmc_split_bf16_transpose": [I64, I64, P, P, I64, P, P, S],
    "hmc_tc_gradient": [I64, I64, I64, P, P, I64, P, P, I64, P, P, I, P, S],
    "hmc_tc_step": [P, P, P, I64, P, P, P, P, I64, P, P, I, P, P, D, D, P, S],
    "hmc_tc_step_split": [P, P, P, I64, P, P, P, P, I64, P, P, I, P, P, D, D, P, S],
    "hmc_tc_resid_misfit": [I64, I64, I64, P, P, I64, P, P, I64, P, P, P, P, I, P, S],
    "hmc_tc_partials_size": [I64, I64],
    "hmc_tc_mlp": [I, I64, I64, I64, P, I64, P, I64, P, P, P, S],
    "hmc_mlp_input": [I64, I64, P, P, P, P, I64, S],
    "hmc_mlp_gather": [I64, I64, P, P, P, P, P, P, P, P, I64, P, I64, P, I64, S],
    "hmc_mlp_loss": [I64, I64, P, I64, P, I64, P, I64, P, I64, P, S],
    "hmc_mlp_bias_grad": [I64, I64, P, I64, P, S],
    "hmc_mlp_adam": [I64, P, P, P, P, _ct.c_float, _ct.c_float, _ct.c_float, _ct.c_float, I64, S],
    "hmc_mlp_cast": [I64, I64, P, P, I64, P, I64, S],
    "hmc_mlp_record": [I64, I64, P, P, I64, S],
    "hmc_pot_elementwise": [I, I64, I64, P, I64, P, I64, P, I64, P, P, I64, P, I64, P, I64, S],
    "hmc_pot_w3_grad": [I64, I64, P, I64, P, I64, P, S],
    "hmc_pot_loss": [I64, I64, P, I64, P, I64, P, P, I64, P, I64, P, S],
    "hmc_pot_scaled_cast": [I64, I64, P, I64, I, P, P, I64, I64, S],
    "hmc_pot_value_residual": [I64, I64, P, I64, P, P, P, _ct.c_float, P, P, S],
    "hmc_pot_weighted_colsum": [I64, I64, P, I64, P, P, S],
    "hmc_pot_scale_columns": [I64, I64, P, I64, P, P, I64, S],
    "hmc_fwi_prepare": [P, S],
    "hmc_fwi_forward_shot": [P, I, I, I, I, S],
    "hmc_fwi_forward_shot_sources": [P, I, P, I, I, S],
    "hmc_fill_zero": [P, I64, S],
    "hmc_fwi_cell_model": [I64, I64, P, P, P, P, S],
    "hmc_fwi_cell_gradient": [I64, I64, P, P, P, P, I, S],
    "hmc_fwi_misfit": [P, I, P, I, S],
    "hmc_fwi_zero_gradients": [P, S],
    "hmc_fwi_adjoint_shot": [P, I, S],
    "hmc_fwi_param_gradient": [P, P, P, P, I, S],
    "hmc_ess": [I, I64, I64, I64, P, I, P, P, P, S],
    "hmc_ess_work_size": [I64, I64, I],
    "hmc_moments": [I, I64, I64, I64, P, P, P, S],
    "hmc_rank_normalize": [I, I64, I64, I64, P, P, S],
    "hmc_graph_begin": [S],
    "hmc_graph_end": [S, _ct.POINTER(c_void_p)],
    "hmc_graph_launch": [P, S],
    "hmc_graph_destroy": [P],
}
_RESTYPES = {
    "hmc_last_error": c_char_p,
    "hmc_launch_count": c_int64,
    "hmc_ess_work_size": c_int64,
    "hmc_tc_partials_size": c_int64,
}

_lock = _threading.Lock()
_lib = None


def library_available():
    return _os.path.exists(LIB_PATH)


def load():
    """Load the shared library once; raise DeviceUnavailableError if absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not _os.path.exists(LIB_PATH):
            raise DeviceUnavailableError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(hmclab_gb300 has no CPU fallback)"
            )
        lib = _ct.CDLL(LIB_PATH)
        for name, argtypes in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = _RESTYPES.get(name, c_int)
        _lib = lib
    return _lib


def last_error():
    return load().hmc_last_error().decode(errors="replace")


def check(rc, name):
    """Map a C status code to the exception class the reference raises."""
    if rc == HMC_OK:
        return
    msg = f"{name}: {last_error()}"
    if rc == HMC_ERR_INVALID_ARG:
        raise ValueError(msg)
    if rc == HMC_ERR_TIMEOUT:
        raise DeviceTimeoutError(msg)
    if rc == HMC_ERR_NONFINITE:
        raise FloatingPointError(msg)
    if rc == HMC_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise RuntimeError(msg)


def call(name, *args):
    rc = getattr(load(), name)(*args)
    check(rc, name)


def launch_count():
    return int(load().hmc_launch_count())


class wait_limits:
    """Context manager around hmc_set_wait_limits (a test hook): inside it,
    bounded device waits give up after `wait_ns`, and with `withhold` block 0
    of every launch that stages tiles through tensor-copy barriers skips its
    arrival, so its wait runs out and the kernel reports a time-out.  The
    production limits (2 s, nothing withheld) are restored on exit."""

    DEFAULT_NS = 2_000_000_000

    def __init__(self, wait_ns, withhold=False):
        self.wait_ns, self.withhold = int(wait_ns), int(bool(withhold))

    def __enter__(self):
        call("hmc_set_wait_limits", self.wait_ns, self.withhold)
        return self

    def __exit__(self, *exc):
        call("hmc_set_wait_limits", self.DEFAULT_NS, 0)
        return False
