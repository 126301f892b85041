"""Host side of the FP32 CSR products of the sparse LinearMatrix.

`CsrSlabPlan` holds, for one sparse LinearMatrix and a chain count C, the
launch shape the autotuner picked for G and for G^T — a gather kernel (one
or four chains per thread) or the shared-memory column-slab kernel with its
slab width and rows per warp, with the slab pointers it needs — and issues
hmc_csr_slab_misfit / hmc_csr_slab_gradient (csrc/distributions.cu).  Every
shape adds a row's nonzeros in CSR order, so all give the same sums bit for
bit; the shape only changes the speed.

Centring: the residual G m - d of a travel-time problem is about a thousandth
of G m, so forming it from FP32 sums of G m would lose three digits.  The
plan centres the products on the minimum-norm least-squares point c of
G c = d: the device forms G (m - c) - (d - G c), with d - G c computed once in
FP64, which leaves the residual unchanged and its FP32 error at the level of
the residual itself.
"""
import numpy as _np

from hmclab_gb300 import _device as _dev
from hmclab_gb300 import _lib
from hmclab_gb300 import autotune as _autotune

SLABS = (128, 192, 256, 320, 384, 448)
ROWS_PER_WARP = (4, 8, 16)


def candidates(C):
    """Launch shapes (kernel, slab, rows per warp) the autotuner times: the
    per-nonzero gather kernels (one or four chains per thread) and the
    shared-memory slab kernel's shapes."""
    out = [(_lib.HMC_CSR_GATHER, 0, 0)]
    if C % 4 == 0:
        out.append((_lib.HMC_CSR_GATHER4, 0, 0))
    out += [(_lib.HMC_CSR_SLAB, s, r) for s in SLABS for r in ROWS_PER_WARP]
    return out


def slab_pointers(indptr, indices, cols, slab):
    """[rows][n_slabs + 1] int32: entry (r, s) is the first nonzero of row r
    whose column is >= s * slab; columns must be sorted within rows."""
    indptr = _np.asarray(indptr, _np.int64)
    indices = _np.asarray(indices, _np.int64)
    rows = len(indptr) - 1
    n_slabs = -(-int(cols) // int(slab))
    row_of = _np.repeat(_np.arange(rows), _np.diff(indptr))
    counts = _np.bincount(row_of * n_slabs + indices // slab, minlength=rows * n_slabs).reshape(rows, n_slabs)
    sp = _np.empty((rows, n_slabs + 1), _np.int64)
    sp[:, 0] = indptr[:-1]
    sp[:, 1:] = indptr[:-1, None] + _np.cumsum(counts, axis=1)
    return sp.astype(_np.int32)


def columns_sorted(indptr, indices):
    """Whether the column indices increase strictly within every row."""
    indptr = _np.asarray(indptr, _np.int64)
    step = _np.diff(_np.asarray(indices, _np.int64))
    if step.size == 0:
        return True
    # positions where a new row starts may step down
    starts = indptr[1:-1] - 1
    ok = step > 0
    ok[starts[(starts >= 0) & (starts < step.size)]] = True
    return bool(ok.all())


class _Matrix:
    """One CSR operand (G or G^T) on the device with its slab pointers."""

    def __init__(self, indptr, indices, rp_dev, col_dev, val_dev, rows, cols, device):
        if not columns_sorted(indptr, indices):
            raise ValueError("the slab CSR products need column indices sorted within rows")
        self.indptr, self.indices = indptr, indices
        self.rp, self.col, self.val = rp_dev, col_dev, val_dev
        self.rows, self.cols, self.device = int(rows), int(cols), device
        self._sp = {}

    def descriptor(self, kernel, slab=0, rpw=0):
        d = _lib.HmcCsrSlabs()
        d.col, d.val, d.row_ptr = self.col.data_ptr(), self.val.data_ptr(), self.rp.data_ptr()
        d.rows, d.cols, d.kernel = self.rows, self.cols, int(kernel)
        if kernel == _lib.HMC_CSR_SLAB:
            sp = self._sp.get(slab)
            if sp is None:
                sp = _dev.upload_int32(slab_pointers(self.indptr, self.indices, self.cols, slab), self.device)
                self._sp[slab] = sp
            d.slab_ptr, d.slab, d.rows_per_warp = sp.data_ptr(), int(slab), int(rpw)
        return d

    def keep_only(self, shape):
        self._sp = {shape[1]: self._sp[shape[1]]} if shape[0] == _lib.HMC_CSR_SLAB else {}


class CsrSlabPlan:
    """The slab products of one sparse LinearMatrix for C chains."""

    def __init__(self, lik, C, device, stream):
        import torch

        p = lik._params("float32")
        G = lik.G
        Gt = lik.G.T.tocsr()
        Gt.sort_indices()
        n, d = lik.n_data, lik.dimensions
        self.C = int(C)
        self.p = p
        self.g = _Matrix(G.indptr, G.indices, p["rp"], p["col"], p["val"], n, d, device)
        self.gt = _Matrix(Gt.indptr, Gt.indices, p["trp"], p["tcol"], p["tval"], d, n, device)
        # autotune each product on zero operands (the timing does not depend on values)
        X = torch.zeros((d, self.C), dtype=torch.float32, device=device)
        R = torch.zeros((n, self.C), dtype=torch.float32, device=device)
        out_n = torch.empty((n, self.C), dtype=torch.float32, device=device)
        out_d = torch.empty((d, self.C), dtype=torch.float32, device=device)
        x = torch.empty((self.C,), dtype=torch.float64, device=device)
        shapes = candidates(self.C)
        nnz = int(G.nnz)

        zeros_d = torch.zeros((d,), dtype=torch.float32, device=device)
        ones_d = torch.ones((d,), dtype=torch.float32, device=device)

        # each product is timed through the misfit entry point (product, then
        # the same per-chain reduction for every candidate)
        def run_g(cand):
            _lib.call("hmc_csr_slab_misfit", _lib._ct.byref(self.g.descriptor(*cand)), self.C, X.data_ptr(),
                      None, p["data"].data_ptr(), p["iv"].data_ptr(), out_n.data_ptr(), x.data_ptr(), 0, stream)

        def run_gt(cand):
            _lib.call("hmc_csr_slab_misfit", _lib._ct.byref(self.gt.descriptor(*cand)), self.C, R.data_ptr(),
                      None, zeros_d.data_ptr(), ones_d.data_ptr(), out_d.data_ptr(), x.data_ptr(), 0, stream)

        # centre of the FP32 products (see the module note)
        import scipy.sparse.linalg as _spla

        dv = _np.asarray(lik.d, _np.float64)[:, 0]
        c = _spla.lsqr(G, dv, atol=1e-12, btol=1e-12, iter_lim=10 * max(n, d))[0]
        c32 = c.astype(_np.float32).astype(_np.float64)
        self.center = _dev.upload(c32, "float32", device)
        self.data_c = _dev.upload(dv - G @ c32, "float32", device)
        self.shape_g = _autotune.choose("csr_slab", {"rows": n, "cols": d, "nnz": nnz, "C": self.C}, shapes, run_g,
                                        device, stream)
        self.shape_gt = _autotune.choose("csr_slab", {"rows": d, "cols": n, "nnz": nnz, "C": self.C}, shapes, run_gt,
                                         device, stream)
        self.desc_g = self.g.descriptor(*self.shape_g)
        self.desc_gt = self.gt.descriptor(*self.shape_gt)
        self.g.keep_only(self.shape_g)
        self.gt.keep_only(self.shape_gt)
        self._ref_g = _lib._ct.byref(self.desc_g)
        self._ref_gt = _lib._ct.byref(self.desc_gt)
        torch.cuda.current_stream(device).synchronize()

    def misfit(self, M, resid, out, accumulate, stream):
        _lib.call("hmc_csr_slab_misfit", self._ref_g, self.C, M.data_ptr(), self.center.data_ptr(),
                  self.data_c.data_ptr(), self.p["iv"].data_ptr(), resid.data_ptr(), out.data_ptr(), int(accumulate),
                  stream)

    def gradient(self, M, resid, out, accumulate, stream):
        _lib.call("hmc_csr_slab_gradient", self._ref_g, self._ref_gt, self.C, M.data_ptr(), self.center.data_ptr(),
                  self.data_c.data_ptr(), self.p["iv"].data_ptr(), resid.data_ptr(), out.data_ptr(), int(accumulate),
                  stream)
