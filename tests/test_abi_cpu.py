"""CPU-side checks of the C ABI: the library loads, exports every function
include/hmclab_gb300.h declares, and the ctypes mirror of `hmc_chains` has the
C layout.  No compute call is made (no GPU here)."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from hmclab_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hmclab_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"HMC_API\s+[\w\s\*]+?\b(hmc_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not _lib.library_available():
        from hmclab_gb300 import build

        build.build()
    return _lib.load()


def test_header_declares_functions():
    names = declared_functions()
    assert "hmc_begin_trajectory" in names and "hmc_end_trajectory" in names
    assert len(names) >= 25


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} is declared in the header but not exported"


def test_python_signatures_cover_header():
    assert set(declared_functions()) == set(_lib.SIGNATURES), (
        "ctypes signatures and header declarations differ: "
        f"{set(declared_functions()) ^ set(_lib.SIGNATURES)}"
    )


def test_version_and_error_string_without_gpu(lib):
    assert lib.hmc_version() == 1
    assert isinstance(lib.hmc_last_error(), bytes)


def test_invalid_arguments_fail_before_any_launch(lib):
    # Null state: rejected on the host, no CUDA call is made.
    rc = lib.hmc_begin_trajectory(None, 0.5, None)
    assert rc == _lib.HMC_ERR_INVALID_ARG
    assert b"null state" in lib.hmc_last_error()
    with pytest.raises(ValueError):
        _lib.check(rc, "hmc_begin_trajectory")
    st = _lib.HmcChains()
    st.dtype = 7
    rc = lib.hmc_end_trajectory(ctypes.byref(st), None)
    assert rc == _lib.HMC_ERR_INVALID_ARG


@pytest.mark.parametrize("cname, cls", [("hmc_chains", _lib.HmcChains), ("hmc_fwi", _lib.HmcFwi),
                                         ("hmc_mlp_out", _lib.HmcMlpOut), ("hmc_schedule", _lib.HmcSchedule),
                                         ("hmc_dense_group", _lib.HmcDenseGroup),
                                         ("hmc_csr_slabs", _lib.HmcCsrSlabs),
                                         ("hmc_fwi_source", _lib.HmcFwiSource)])
def test_struct_layout_matches_c(tmp_path, cname, cls):
    """Compile a probe with gcc that prints sizeof/offsetof of the C struct
    and compare with the ctypes Structure."""
    fields = [f for f, _ in cls._fields_]
    src = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){",
           f'printf("%zu\\n", sizeof({cname}));']
    for f in fields:
        src.append(f'printf("%zu\\n", offsetof({cname}, {f}));')
    src.append("return 0;}")
    c = tmp_path / "probe.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-o", str(exe), str(c)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(cls)
    for f, off in zip(fields, out[1:]):
        assert getattr(cls, f).offset == off, f


def test_new_entry_points_reject_bad_arguments_on_the_host(lib):
    """Argument checks of the potential-surrogate, rank-normalisation and
    FWI entry points run before any CUDA call (no GPU here)."""
    E = _lib.HMC_ERR_INVALID_ARG
    # unknown element-wise mode, missing buffers, bad pitches
    assert lib.hmc_pot_elementwise(9, 4, 4, None, 0, ctypes.c_void_p(8), 4, None, 0, None, ctypes.c_void_p(8), 4,
                                   None, 0, None, 0, None) == E
    assert b"unknown mode" in lib.hmc_last_error()
    assert lib.hmc_pot_elementwise(_lib.HMC_POT_DELTA2, 4, 4, None, 0, ctypes.c_void_p(8), 4, None, 0, None,
                                   ctypes.c_void_p(8), 4, None, 0, None, 0, None) == E
    assert lib.hmc_pot_elementwise(_lib.HMC_POT_DELTA1, 4, 8, ctypes.c_void_p(8), 8, ctypes.c_void_p(8), 4, None, 0,
                                   None, ctypes.c_void_p(8), 8, None, 0, None, 0, None) == E
    assert lib.hmc_pot_loss(4, 8, ctypes.c_void_p(8), 4, ctypes.c_void_p(8), 8, ctypes.c_void_p(8),
                            ctypes.c_void_p(8), 8, ctypes.c_void_p(8), 4, ctypes.c_void_p(8), None) == E
    assert lib.hmc_pot_w3_grad(0, 8, None, 8, None, 8, None, None) == E
    assert lib.hmc_pot_scaled_cast(4, 4, ctypes.c_void_p(8), 4, 0, ctypes.c_void_p(8), ctypes.c_void_p(8), 6, 4,
                                   None) == E
    # the S^2 d comparison budget of the rank normalisation
    assert lib.hmc_rank_normalize(_lib.HMC_F32, 100000, 200, 64, ctypes.c_void_p(8), ctypes.c_void_p(8), None) == E
    assert b"budget" in lib.hmc_last_error()
    assert lib.hmc_rank_normalize(_lib.HMC_F32, 10, 2, 4, None, ctypes.c_void_p(8), None) == E
    # FWI entry points with no descriptor
    assert lib.hmc_fwi_forward_shot(None, 0, 0, 0, 0, None) == E
    assert lib.hmc_fwi_adjoint_shot(None, 0, None) == E


def _fake_fwi():
    """An hmc_fwi whose buffers are non-null placeholders: only the host-side
    validation below may look at it (every case fails before a launch)."""
    s = _lib.HmcFwi()
    s.nx, s.nz, s.nt, s.nrec, s.chains = 40, 30, 10, 3, 32
    s.h, s.dt, s.w = 5.0, 5e-4, 1.0
    dummy = 0x1000
    for name in ("taper", "stf_host", "rec_map", "rho", "vp", "vs", "bx", "bz", "l2m", "lam", "muxz", "vx", "vz",
                 "sxx", "szz", "sxz", "rec"):
        setattr(s, name, dummy)
    return s


def test_fwi_source_validation_happens_on_the_host(lib):
    s = _fake_fwi()
    stf = (ctypes.c_float * 10)()

    def sources(n, x=10, z=10, mxz=0.0, wavelet=True):
        arr = (_lib.HmcFwiSource * n)()
        for k in range(n):
            arr[k].x, arr[k].z = x, z
            arr[k].mxx, arr[k].mzz, arr[k].mxz = 1.0, 1.0, mxz
            arr[k].stf_host = ctypes.cast(stf, ctypes.c_void_p).value if wavelet else None
        return arr

    for arr, why in ((sources(9, mxz=0.5), "stress terms"), (sources(1, x=0), "interior"),
                     (sources(1, z=30), "interior"), (sources(1, wavelet=False), "wavelet")):
        rc = lib.hmc_fwi_forward_shot_sources(ctypes.byref(s), 0, arr, len(arr), 0, None)
        assert rc == _lib.HMC_ERR_INVALID_ARG
        assert why in _lib.last_error()
    rc = lib.hmc_fwi_forward_shot_sources(ctypes.byref(s), 0, None, 0, 0, None)
    assert rc == _lib.HMC_ERR_INVALID_ARG
    # storing for the adjoint needs the store buffer
    rc = lib.hmc_fwi_forward_shot_sources(ctypes.byref(s), 0, sources(2), 2, 1, None)
    assert rc == _lib.HMC_ERR_INVALID_ARG and "store" in _lib.last_error()


def test_cell_parametrisation_and_fill_reject_bad_sizes(lib):
    assert lib.hmc_fwi_cell_model(0, 4, None, None, None, None, None) == _lib.HMC_ERR_INVALID_ARG
    assert lib.hmc_fwi_cell_gradient(5, 0, None, None, None, None, 0, None) == _lib.HMC_ERR_INVALID_ARG
    assert lib.hmc_fill_zero(None, -1, None) == _lib.HMC_ERR_INVALID_ARG
    assert lib.hmc_fill_zero(None, 0, None) == _lib.HMC_OK
