"""Shared-memory column-slab CSR products (csrc/distributions.cu,
hmclab_gb300/_csr.py) and the launch-shape autotuner (autotune.py).

CPU: slab pointers partition every row by column slab; the sortedness check;
the autotuner's cache file.  GPU: every launch shape (the gather kernels with
one or four chains per thread, the slab kernel's shapes) gives the same FP32
misfits and gradients as hmc_csr_misfit / hmc_csr_gradient bit for bit, and
the centred public path matches the FP64 host product within the FP32
parity tolerance (1e-5 of the largest |gradient| entry)."""
import json

import numpy as np
import pytest
import scipy.sparse as sp

from hmclab_gb300 import _csr
from hmclab_gb300 import autotune


def _random_csr(rows, cols, density, seed):
    G = sp.random(rows, cols, density=density, format="csr", random_state=seed, dtype=np.float64)
    G.sort_indices()
    return G


@pytest.mark.parametrize("slab", [32, 64, 100, 4096])
def test_slab_pointers_partition_rows(slab):
    G = _random_csr(70, 777, 0.05, 3)
    P = _csr.slab_pointers(G.indptr, G.indices, 777, slab)
    n_slabs = -(-777 // slab)
    assert P.shape == (70, n_slabs + 1)
    for r in range(70):
        assert P[r, 0] == G.indptr[r] and P[r, -1] == G.indptr[r + 1]
        assert np.all(np.diff(P[r]) >= 0)
        for s in range(n_slabs):
            seg = G.indices[P[r, s]:P[r, s + 1]]
            assert np.all((seg >= s * slab) & (seg < (s + 1) * slab))


def test_columns_sorted_detects_unsorted_rows():
    G = _random_csr(20, 50, 0.3, 1)
    assert _csr.columns_sorted(G.indptr, G.indices)
    idx = G.indices.copy()
    r = int(np.argmax(np.diff(G.indptr) >= 2))
    a, b = G.indptr[r], G.indptr[r + 1]
    idx[a:b] = idx[a:b][::-1]
    assert not _csr.columns_sorted(G.indptr, idx)
    # empty rows and a single row are sorted
    assert _csr.columns_sorted(np.array([0, 0, 0]), np.array([], np.int32))


def test_autotune_cache_file_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "shapes.json"
    monkeypatch.setenv("HMCLAB_GB300_TUNE_CACHE", str(path))
    assert autotune.cache_path() == str(path)
    autotune._write(str(path), "dev|k|{}", {"choice": [512, 8], "ms": {"512,8": 0.1}})
    autotune._write(str(path), "dev|k2|{}", {"choice": [256, 4]})
    data = json.loads(path.read_text())
    assert data["dev|k|{}"]["choice"] == [512, 8] and data["dev|k2|{}"]["choice"] == [256, 4]
    monkeypatch.setenv("HMCLAB_GB300_TUNE_CACHE", "")
    assert autotune.cache_path() is None
    path.write_text("not json")
    assert autotune._read(str(path)) == {}


# ---------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("rows,cols,C", [(2000, 4096, 1024), (300, 700, 77), (513, 129, 33), (5, 3000, 1)])
def test_slab_products_equal_gather_kernels(rows, cols, C):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import hmclab_gb300 as H
    from hmclab_gb300 import _lib

    rng = np.random.default_rng(rows + cols)
    G = _random_csr(rows, cols, min(0.05, 130.0 / cols), rows)
    G.data = rng.uniform(0.0, 1.5, size=G.nnz)
    dat = rng.normal(size=(rows, 1))
    lik = H.Distributions.LinearMatrix(G, dat, 0.01, premultiplication=False)
    assert not lik.dense and not lik.premultiplication
    M = torch.from_numpy(rng.normal(size=(cols, C))).to("cuda", torch.float32)
    p = lik._params("float32")
    h = torch.cuda.current_stream().cuda_stream
    resid = torch.empty((rows, C), dtype=torch.float32, device="cuda")
    g_old = torch.empty((cols, C), dtype=torch.float32, device="cuda")
    x_old = torch.empty((C,), dtype=torch.float64, device="cuda")
    _lib.call("hmc_csr_gradient", _lib.HMC_F32, rows, cols, C, M.data_ptr(), p["rp"].data_ptr(), p["col"].data_ptr(),
              p["val"].data_ptr(), p["trp"].data_ptr(), p["tcol"].data_ptr(), p["tval"].data_ptr(),
              p["data"].data_ptr(), p["iv"].data_ptr(), resid.data_ptr(), g_old.data_ptr(), 0, h)
    _lib.call("hmc_csr_misfit", _lib.HMC_F32, rows, cols, C, M.data_ptr(), p["rp"].data_ptr(), p["col"].data_ptr(),
              p["val"].data_ptr(), p["data"].data_ptr(), p["iv"].data_ptr(), resid.data_ptr(), x_old.data_ptr(), 0, h)
    plan = lik._csr_plan(C, M.device, h)
    shapes = [c for c in _csr.candidates(C) if c[0] != _lib.HMC_CSR_SLAB or c[1] in _csr.SLABS[::2]]
    shapes += [(_lib.HMC_CSR_SLAB, 32, r) for r in _csr.ROWS_PER_WARP]
    for shape in shapes:
        dg, dgt = plan.g.descriptor(*shape), plan.gt.descriptor(*shape)
        g = torch.full((cols, C), float("nan"), dtype=torch.float32, device="cuda")
        x = torch.empty((C,), dtype=torch.float64, device="cuda")
        _lib.call("hmc_csr_slab_gradient", _lib._ct.byref(dg), _lib._ct.byref(dgt), C, M.data_ptr(), None,
                  p["data"].data_ptr(), p["iv"].data_ptr(), resid.data_ptr(), g.data_ptr(), 0, h)
        _lib.call("hmc_csr_slab_misfit", _lib._ct.byref(dg), C, M.data_ptr(), None, p["data"].data_ptr(),
                  p["iv"].data_ptr(), resid.data_ptr(), x.data_ptr(), 0, h)
        torch.cuda.synchronize()
        assert torch.equal(g, g_old), shape
        assert torch.equal(x, x_old), shape
    # the public path (autotuned shape, centred products) and the FP64 host product
    g = lik.gradient_batch(M).double().cpu().numpy()
    x = lik.misfit_batch(M).cpu().numpy()
    Mh = M.double().cpu().numpy()
    r64 = lik.G @ Mh - lik.d
    g64 = lik.G.T @ (r64 * lik.inv_var)
    x64 = 0.5 * np.sum(r64 * r64 * lik.inv_var, axis=0)
    err = np.abs(g - g64).max() / np.abs(g64).max()
    xerr = np.max(np.abs(x - x64) / x64)
    print(f"{rows}x{cols} C={C}: slab shapes {plan.shape_g} / {plan.shape_gt}, FP32 vs FP64 gradient {err:.2e}, "
          f"misfit {xerr:.2e}")
    assert err < 1e-5 and xerr < 1e-5


@pytest.mark.gpu
def test_centred_products_hold_the_tomography_misfit_to_fp32_precision():
    """Travel times ~1e3 x their residuals: without centring the FP32 misfit
    loses about three digits; the centred products keep it near 1e-6."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bench

    wl = bench.TomoWorkload(seed=0)
    post = wl.posterior()
    lik = post.separate_distributions[1]
    M = torch.from_numpy(wl.q0[:, :256]).to("cuda", torch.float32)
    x = lik.misfit_batch(M).cpu().numpy()
    Mh = M.double().cpu().numpy()
    r64 = lik.G @ Mh - lik.d
    x64 = 0.5 * np.sum(r64 * r64 * lik.inv_var, axis=0)
    xerr = np.max(np.abs(x - x64) / x64)
    print(f"tomography misfit, 256 posterior draws: FP32 centred vs FP64 {xerr:.2e} (misfit ~{np.median(x64):.0f})")
    assert xerr < 2e-6
