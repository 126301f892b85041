"""Learned gradient surrogate for HMC: a d-512-512-d GELU MLP with BF16
weights and activations and FP32 accumulation, trained on the GPU by the
project's own kernels (tensor-core contractions in csrc/dense_tc.cu, Adam and
data movement in csrc/mlp.cu).

Exactness: the sampler uses the surrogate only for the interior kicks of the
leapfrog (the `distribution.gradient` calls of Samplers.py:1562,1573 in the
reference); the exact misfit at the trajectory end decides acceptance.  Any
fixed force field keeps the leapfrog volume-preserving and reversible, so the
chain still targets the exact posterior as long as the network is frozen
while samples are collected (it is trained during burn-in, then frozen).

Normalisation: inputs x = (q - mu_q) / sigma_q, targets
y = (grad U - mu_g) / sigma_g (per coordinate, from the training set); the
loss is 0.5 * mean over the batch of |f(x) - y|^2.

Architecture: h1 = GELU(W1 x + b1), h2 = GELU(W2 h1 + b2),
f(x) = W3 [h2 | x] + b3 — the output layer also sees the input (a linear
skip path), initialised to the least-squares linear fit of the training set,
so the hidden layers learn the nonlinear part of the gradient field.  The
input is stored inside the output layer's activation buffer, so the skip
costs no extra launch.
"""
import numpy as _np

from hmclab_gb300 import _device as _dev
from hmclab_gb300 import _lib


def _pad(n):
    return (int(n) + 63) // 64 * 64


class TrainingSet:
    """Device stores of (position, exact gradient) pairs, [capacity][d] FP32."""

    def __init__(self, dimensions, capacity, device=None):
        import torch

        device = device or _dev.require_cuda()
        self.d, self.capacity = int(dimensions), int(capacity)
        self.q = torch.zeros((self.capacity, self.d), dtype=torch.float32, device=device)
        self.g = torch.zeros_like(self.q)
        self.count = 0

    def record(self, q, g, stream):
        """Append the columns of q, g ([d][C] device tensors) as C new rows."""
        C = q.shape[1]
        if self.count + C > self.capacity:
            return False
        _lib.call("hmc_mlp_record", self.d, C, q.data_ptr(), self.q.data_ptr(), self.count, stream)
        _lib.call("hmc_mlp_record", self.d, C, g.data_ptr(), self.g.data_ptr(), self.count, stream)
        self.count += C
        return True


class MLPSurrogate:
    def __init__(self, dimensions, hidden=(512, 512), seed=0, device=None):
        import torch

        self.device = device or _dev.require_cuda()
        self.d = int(dimensions)
        self.sizes = [self.d, int(hidden[0]), int(hidden[1]), self.d]
        # the input sits after the second hidden layer in one BF16 row: keep it
        # on a 16-element (32-byte) boundary for the tensor-memory copies
        assert self.sizes[1] % 16 == 0 and self.sizes[2] % 16 == 0, "hidden widths must be multiples of 16"
        rng = _np.random.default_rng(seed)
        f32 = dict(dtype=torch.float32, device=self.device)
        self.W, self.b, self.mW, self.vW, self.mb, self.vb, self.gW, self.gb = ([] for _ in range(8))
        self.W16, self.W16t = [], []
        self.k3 = self.sizes[2] + self.d  # output layer reads [h2 | x]
        # weights and biases uniform in +-1/sqrt(fan_in) (the output layer's
        # hidden block 10x smaller): the larger He-normal scale with zero
        # biases fits the training pairs equally well but generalises
        # several times worse between them
        for l in range(3):
            n_in, n_out = (self.sizes[l] if l < 2 else self.k3), self.sizes[l + 1]
            bound = (1.0 / n_in) ** 0.5 * (1.0 if l < 2 else 0.1)
            self.W.append(torch.from_numpy(rng.uniform(-bound, bound, size=(n_out, n_in))).to(**f32).contiguous())
            self.b.append(torch.from_numpy(rng.uniform(-bound, bound, size=n_out) if l < 2 else _np.zeros(n_out))
                          .to(**f32))
            for lst, shape in ((self.mW, (n_out, n_in)), (self.vW, (n_out, n_in)), (self.gW, (n_out, n_in)),
                               (self.mb, (n_out,)), (self.vb, (n_out,)), (self.gb, (n_out,))):
                lst.append(torch.zeros(shape, **f32))
            self.W16.append(torch.zeros((n_out, _pad(n_in)), dtype=torch.bfloat16, device=self.device))
            self.W16t.append(torch.zeros((n_in, _pad(n_out)), dtype=torch.bfloat16, device=self.device))
        self.mu_q = torch.zeros(self.d, **f32)
        self.inv_q = torch.ones(self.d, **f32)
        self.mu_g = torch.zeros(self.d, **f32)
        self.sig_g = torch.ones(self.d, **f32)
        self.inv_g = torch.ones(self.d, **f32)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.loss_buf = torch.zeros(1025, dtype=torch.float64, device=self.device)
        self.steps = 0
        self._bufs = {}
        self._cast(_dev.stream_handle())
        self.frozen = False

    # ---- buffers ---------------------------------------------------------
    def _buffers(self, B, training):
        import torch

        key = (int(B), bool(training))
        if key in self._bufs:
            return self._bufs[key]
        bf, f32 = torch.bfloat16, torch.float32
        dev = self.device
        d, h1, h2 = self.sizes[0], self.sizes[1], self.sizes[2]
        pB = _pad(B)
        z = lambda shape, dt: torch.zeros(shape, dtype=dt, device=dev)  # noqa: E731
        # A2 holds [h2 | x] per row: the second hidden activations and the input
        A2 = z((B, _pad(self.k3)), bf)
        A2t = z((self.k3, pB), bf)
        b = {
            "A2": A2, "A2t": A2t,
            "X": A2[:, h2:], "Xt": A2t[h2:],
            "Z1": z((B, h1), f32), "A1": z((B, _pad(h1)), bf), "A1t": z((h1, pB), bf),
            "Z2": z((B, h2), f32),
        }
        if training:
            b.update({
                "idx": z((B,), torch.int32), "T": z((B, d), f32), "Y": z((B, d), f32),
                "dY": z((B, _pad(d)), bf), "dYt": z((d, pB), bf),
                "dZ2": z((B, _pad(h2)), bf), "dZ2t": z((h2, pB), bf),
                "dZ1": z((B, _pad(h1)), bf), "dZ1t": z((h1, pB), bf),
            })
        self._bufs[key] = b
        return b

    def _cast(self, stream):
        for l in range(3):
            n_out, n_in = self.W[l].shape
            _lib.call("hmc_mlp_cast", n_out, n_in, self.W[l].data_ptr(), self.W16[l].data_ptr(), _pad(n_in),
                      self.W16t[l].data_ptr(), _pad(n_out), stream)

    def _out(self, **kw):
        o = _lib.HmcMlpOut()
        for k, v in kw.items():
            setattr(o, k, v.data_ptr() if hasattr(v, "data_ptr") else v)
        return o

    def _mm(self, mode, M, N, K, x, ldx, l, bias, out, stream, transposed_w=False):
        import ctypes

        w = self.W16t[l] if transposed_w else self.W16[l]
        _lib.call("hmc_tc_mlp", mode, M, N, K, x.data_ptr(), ldx, w.data_ptr(), w.shape[1],
                  bias.data_ptr() if bias is not None else None, ctypes.byref(out), self.status.data_ptr(), stream)

    def _forward(self, b, B, stream, g_state=None):
        d, h1, h2 = self.sizes[0], self.sizes[1], self.sizes[2]
        pB = _pad(B)
        lda2 = b["A2"].shape[1]
        o1 = self._out(z=b["Z1"], ldz=h1, act=b["A1"], ld_act=_pad(h1), act_t=b["A1t"], ld_act_t=pB)
        self._mm(_lib.HMC_MLP_HIDDEN, B, h1, d, b["X"], lda2, 0, self.b[0], o1, stream)
        o2 = self._out(z=b["Z2"], ldz=h2, act=b["A2"], ld_act=lda2, act_t=b["A2t"], ld_act_t=pB)
        self._mm(_lib.HMC_MLP_HIDDEN, B, h2, h1, b["A1"], _pad(h1), 1, self.b[1], o2, stream)
        if g_state is None:
            o3 = self._out(y=b["Y"], ldy=d)
        else:
            o3 = self._out(g_state=g_state, out_scale=self.sig_g, out_shift=self.mu_g)
        self._mm(_lib.HMC_MLP_OUT, B, d, self.k3, b["A2"], lda2, 2, self.b[2], o3, stream)

    # ---- normalisation ---------------------------------------------------
    def fit_normalization(self, data: TrainingSet, rows=None):
        """Per-coordinate input/target normalisation and the least-squares
        start of the linear skip, from the stored pairs (or the given rows)."""
        import torch

        n = data.count
        if rows is None:
            q = data.q[:n].double()
            g = data.g[:n].double()
        else:
            r = torch.as_tensor(_np.asarray(rows), device=self.device)
            q = data.q[r].double()
            g = data.g[r].double()
            n = len(rows)
        sq = q.std(dim=0).clamp_min(1e-12)
        sg = g.std(dim=0).clamp_min(1e-12)
        self.mu_q.copy_(q.mean(dim=0).float())
        self.inv_q.copy_((1.0 / sq).float())
        self.mu_g.copy_(g.mean(dim=0).float())
        self.sig_g.copy_(sg.float())
        self.inv_g.copy_((1.0 / sg).float())
        # linear skip initialised to the ridge least-squares map x -> y
        x = ((q - q.mean(dim=0)) / sq).cpu().numpy()
        y = ((g - g.mean(dim=0)) / sg).cpu().numpy()
        lam = 1e-3 * n
        ws = _np.linalg.solve(x.T @ x + lam * _np.eye(self.d), x.T @ y).T  # [d_out][d_in]
        h2 = self.sizes[2]
        self.W[2][:, h2:] = torch.from_numpy(ws).float().to(self.device)
        self._cast(_dev.stream_handle())
        torch.cuda.synchronize(self.device)

    # ---- training --------------------------------------------------------
    def train_step(self, data: TrainingSet, idx_host, lr=1e-3, stream=None, beta1=0.9, beta2=0.999, eps=1e-8):
        """One Adam step on the minibatch rows idx_host; returns the device
        loss buffer (loss_buf[0] = 0.5 * mean |f(x) - y|^2)."""
        import torch

        assert not self.frozen, "the surrogate is frozen"
        h = _dev.stream_handle(stream)
        B = len(idx_host)
        b = self._buffers(B, True)
        d, h1, h2 = self.sizes[0], self.sizes[1], self.sizes[2]
        pB = _pad(B)
        b["idx"].copy_(torch.from_numpy(_np.asarray(idx_host, _np.int32)), non_blocking=False)
        _lib.call("hmc_mlp_gather", B, d, b["idx"].data_ptr(), data.q.data_ptr(), data.g.data_ptr(),
                  self.mu_q.data_ptr(), self.inv_q.data_ptr(), self.mu_g.data_ptr(), self.inv_g.data_ptr(),
                  b["X"].data_ptr(), b["A2"].shape[1], b["Xt"].data_ptr(), pB, b["T"].data_ptr(), d, h)
        self._forward(b, B, h)
        _lib.call("hmc_mlp_loss", B, d, b["Y"].data_ptr(), d, b["T"].data_ptr(), d, b["dY"].data_ptr(), _pad(d),
                  b["dYt"].data_ptr(), pB, self.loss_buf.data_ptr(), h)
        # layer 3 (its input is [h2 | x])
        self._wgrad(self.k3, d, B, b["A2t"], pB, b["dYt"], 2, h)
        _lib.call("hmc_mlp_bias_grad", d, B, b["dYt"].data_ptr(), pB, self.gb[2].data_ptr(), h)
        o = self._out(z=b["Z2"], ldz=h2, act=b["dZ2"], ld_act=_pad(h2), act_t=b["dZ2t"], ld_act_t=pB)
        self._mm(_lib.HMC_MLP_BACK, B, h2, d, b["dY"], _pad(d), 2, None, o, h, transposed_w=True)
        # layer 2
        self._wgrad(h1, h2, B, b["A1t"], pB, b["dZ2t"], 1, h)
        _lib.call("hmc_mlp_bias_grad", h2, B, b["dZ2t"].data_ptr(), pB, self.gb[1].data_ptr(), h)
        o = self._out(z=b["Z1"], ldz=h1, act=b["dZ1"], ld_act=_pad(h1), act_t=b["dZ1t"], ld_act_t=pB)
        self._mm(_lib.HMC_MLP_BACK, B, h1, h2, b["dZ2"], _pad(h2), 1, None, o, h, transposed_w=True)
        # layer 1
        self._wgrad(d, h1, B, b["Xt"], pB, b["dZ1t"], 0, h)
        _lib.call("hmc_mlp_bias_grad", h1, B, b["dZ1t"].data_ptr(), pB, self.gb[0].data_ptr(), h)
        self.steps += 1
        for l in range(3):
            _lib.call("hmc_mlp_adam", self.W[l].numel(), self.W[l].data_ptr(), self.gW[l].data_ptr(),
                      self.mW[l].data_ptr(), self.vW[l].data_ptr(), lr, beta1, beta2, eps, self.steps, h)
            _lib.call("hmc_mlp_adam", self.b[l].numel(), self.b[l].data_ptr(), self.gb[l].data_ptr(),
                      self.mb[l].data_ptr(), self.vb[l].data_ptr(), lr, beta1, beta2, eps, self.steps, h)
        self._cast(h)
        return self.loss_buf

    def _wgrad(self, n_in, n_out, B, act_t, ld_act_t, delta_t, l, stream):
        """gW[l] [n_out][n_in] = sum_b delta[b][out] act[b][in] (K = batch)."""
        import ctypes

        o = self._out(g=self.gW[l], accumulate=0)
        _lib.call("hmc_tc_mlp", _lib.HMC_MLP_WGRAD, n_in, n_out, B, act_t.data_ptr(), ld_act_t, delta_t.data_ptr(),
                  delta_t.shape[1], None, ctypes.byref(o), self.status.data_ptr(), stream)

    def train(self, data: TrainingSet, steps=2000, batch=256, lr=1e-3, seed=0, lr_decay=True, stream=None, rows=None):
        """Fit the network with Adam on the first `rows` pairs of data (all by
        default); returns the loss history (host)."""
        rng = _np.random.default_rng(seed)
        n = data.count if rows is None else min(int(rows), data.count)
        assert n >= batch, "not enough training pairs"
        history = []
        for s in range(steps):
            rate = lr * (0.5 * (1 + _np.cos(_np.pi * s / steps)) if lr_decay else 1.0)
            idx = rng.integers(0, n, size=batch)
            loss = self.train_step(data, idx, lr=float(rate), stream=stream)
            if s % 50 == 0 or s == steps - 1:
                history.append((s, float(loss[0].item())))
        self.check_status()
        return history

    def fit(self, data: TrainingSet, steps=3000, batch=256, lr=1e-3, holdout_fraction=0.1, check_every=200,
            seed=0, stream=None):
        """Train with early stopping: a random `holdout_fraction` of the stored
        pairs is held out, and every `check_every` steps its relative error
        is measured; the weights with the lowest one are kept.  Returns a
        dict with the loss history, the held-out errors (step 0 is the
        least-squares linear start) and the best step."""
        import torch

        n = data.count
        rng = _np.random.default_rng(seed)
        perm = rng.permutation(n)
        n_hold = max(1, int(round(holdout_fraction * n)))
        held = torch.from_numpy(_np.sort(perm[:n_hold])).to(self.device)
        train_rows = _np.sort(perm[n_hold:])
        assert len(train_rows) >= batch, "not enough training pairs"
        self.fit_normalization(data, rows=train_rows)
        err0 = self.relative_error(data, held, stream=stream)
        best = (err0, 0, [w.clone() for w in self.W], [b.clone() for b in self.b])
        errors = [(0, err0)]
        history = []
        done = 0
        while done < steps:
            chunk = min(check_every, steps - done)
            for s in range(chunk):
                k = done + s
                rate = lr * 0.5 * (1 + _np.cos(_np.pi * k / steps))
                idx = train_rows[rng.integers(0, len(train_rows), size=batch)]
                loss = self.train_step(data, idx, lr=float(rate), stream=stream)
                if k % 50 == 0:
                    history.append((k, float(loss[0].item())))
            done += chunk
            e = self.relative_error(data, held, stream=stream)
            errors.append((done, e))
            if e < best[0]:
                best = (e, done, [w.clone() for w in self.W], [b.clone() for b in self.b])
        self.check_status()
        for l in range(3):
            self.W[l].copy_(best[2][l])
            self.b[l].copy_(best[3][l])
        self._cast(_dev.stream_handle(stream))
        torch.cuda.synchronize(self.device)
        return {"history": history, "heldout": errors, "best_step": best[1], "best_heldout": best[0],
                "train_pairs": len(train_rows), "heldout_pairs": n_hold}

    def freeze(self):
        self.frozen = True
        return self

    # ---- inference for the sampler -----------------------------------------
    def predict_into(self, q, g, stream):
        """g [d][C] = surrogate gradient at the chain positions q [d][C]."""
        C = q.shape[1]
        b = self._buffers(C, False)
        _lib.call("hmc_mlp_input", self.d, C, q.data_ptr(), self.mu_q.data_ptr(), self.inv_q.data_ptr(),
                  b["X"].data_ptr(), b["A2"].shape[1], stream)
        self._forward(b, C, stream, g_state=g)

    def relative_error(self, data: TrainingSet, rows, stop=None, stream=None):
        """|f(q) - g| / |g| (Frobenius norms) over stored pairs of data: the
        rows [rows, stop) when `stop` is given, else the index tensor `rows`.
        The held-out error when those pairs were not trained on."""
        import torch

        sel = slice(rows, stop) if stop is not None else rows
        q = data.q[sel].t().contiguous()
        g = data.g[sel].t().contiguous()
        out = torch.empty_like(g)
        self.predict_into(q, out, _dev.stream_handle(stream))
        torch.cuda.synchronize(self.device)
        return float(torch.linalg.norm((out - g).double()) / torch.linalg.norm(g.double()))

    def check_status(self):
        from hmclab_gb300.Helpers.CustomExceptions import DeviceTimeoutError

        s = int(self.status.cpu()[0])
        if s:
            self.status.zero_()
            raise DeviceTimeoutError(f"surrogate contraction reported status {s}")
