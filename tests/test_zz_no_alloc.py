"""hmc_dense_resid_misfit_noalloc: the dense linear misfit for callers that
cannot allocate device memory (their framework owns every device allocation,
or an allocation would stall a latency-critical path).  Its residual lives in
a fixed 16 MiB array inside the library, so it must give the same misfits as
hmc_dense_resid_misfit with a caller-allocated residual buffer, call after
call, even though every call reuses (and overwrites) that one array.

This file is collected last so that a run stopping at its first failure has
already run every other test; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

FP32_RTOL = 1e-5
FP64_RTOL = 1e-12


def _lib_or_skip():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from hmclab_gb300 import _lib

    return _lib, _lib.load()


@pytest.mark.parametrize("dtype,code_name,rtol", [(torch.float64, "HMC_F64", FP64_RTOL), (torch.float32, "HMC_F32", FP32_RTOL)])
def test_noalloc_matches_allocating_entry_point_twice(dtype, code_name, rtol):
    _lib, lib = _lib_or_skip()
    code = getattr(_lib, code_name)
    rng = np.random.default_rng(11)
    n, d, C = 300, 120, 96
    G = torch.from_numpy(rng.normal(size=(n, d)) / np.sqrt(d)).to("cuda", dtype)
    data = torch.from_numpy(rng.normal(size=n)).to("cuda", dtype)
    iv = torch.from_numpy(rng.uniform(0.5, 2.0, size=n)).to("cuda", dtype)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        M = torch.from_numpy(rng.normal(size=(d, C))).to("cuda", dtype)
        ref = torch.zeros(C, dtype=torch.float64, device="cuda")
        resid = torch.empty((n, C), dtype=dtype, device="cuda")
        rc = lib.hmc_dense_resid_misfit(code, n, d, C, M.data_ptr(), G.data_ptr(), data.data_ptr(), iv.data_ptr(),
                                        resid.data_ptr(), ref.data_ptr(), 0, stream)
        assert rc == 0, _lib.last_error()
        out = torch.full((C,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.hmc_dense_resid_misfit_noalloc(code, n, d, C, M.data_ptr(), G.data_ptr(), data.data_ptr(),
                                                iv.data_ptr(), out.data_ptr(), 0, stream)
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), ref.cpu().numpy(), rtol=rtol, err_msg=f"call {call}")
        # and against the misfit in FP64 on the host, from the same (rounded) inputs
        Gh, Mh = G.double().cpu().numpy(), M.double().cpu().numpy()
        r = Gh @ Mh - data.double().cpu().numpy()[:, None]
        x64 = 0.5 * np.sum(r * r * iv.double().cpu().numpy()[:, None], axis=0)
        np.testing.assert_allclose(out.cpu().numpy(), x64, rtol=rtol, err_msg=f"call {call} vs FP64 host misfit")


def test_noalloc_rejects_sizes_beyond_its_scratch():
    _lib, lib = _lib_or_skip()
    n, d = 2048, 8
    C = (16 << 20) // 4 // n + 1  # one chain more than fits in FP32
    dummy = torch.zeros(1, device="cuda")
    out = torch.zeros(C, dtype=torch.float64, device="cuda")
    rc = lib.hmc_dense_resid_misfit_noalloc(_lib.HMC_F32, n, d, C, dummy.data_ptr(), dummy.data_ptr(),
                                            dummy.data_ptr(), dummy.data_ptr(), out.data_ptr(), 0, None)
    assert rc == _lib.HMC_ERR_INVALID_ARG
    assert "exceeds" in _lib.last_error()
