"""Learned gradient surrogates for HMC, with BF16 weights and activations and
FP32 accumulation, trained on the GPU by the project's own kernels
(tensor-core contractions in csrc/dense_tc.cu; Adam and data movement in
csrc/mlp.cu; the potential network's element-wise passes in
csrc/potential.cu):

  PotentialSurrogate  a scalar network f(q) whose gradient drives the
                      leapfrog (a curl-free field), trained by matching its
                      gradient to the exact gradients;
  MLPSurrogate        a d-512-512-d network that outputs the gradient.

The rest of this note describes MLPSurrogate; PotentialSurrogate documents
its own architecture.

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
    """Device stores of (position, exact gradient) pairs, [capacity][d] FP32,
    and with `values=True` the exact misfit at each position ([capacity]
    FP64; the sampler fills it from the forward simulation that precedes
    each exact gradient, where the target offers that)."""

    def __init__(self, dimensions, capacity, device=None, values=False):
        import torch

        device = device or _dev.require_cuda()
        self.d, self.capacity = int(dimensions), int(capacity)
        self.q = torch.zeros((self.capacity, self.d), dtype=torch.float32, device=device)
        self.g = torch.zeros_like(self.q)
        self.x = torch.full((self.capacity,), float("nan"), dtype=torch.float64, device=device) if values else None
        self.count = 0

    @property
    def with_values(self):
        return self.x is not None

    def record(self, q, g, stream, x=None):
        """Append the columns of q, g ([d][C] device tensors) as C new rows
        (and x [C], the misfits at q, when the set keeps values)."""
        import torch

        C = q.shape[1]
        if self.count + C > self.capacity:
            return False
        _lib.call("hmc_mlp_record", self.d, C, q.data_ptr(), self.q.data_ptr(), self.count, stream)
        _lib.call("hmc_mlp_record", self.d, C, g.data_ptr(), self.g.data_ptr(), self.count, stream)
        if self.x is not None and x is not None:
            with torch.cuda.stream(torch.cuda.ExternalStream(stream, device=self.q.device)):
                self.x[self.count:self.count + C].copy_(x)
        self.count += C
        return True


class _Surrogate:
    """Training loop, validation and status checks shared by the surrogates.
    Subclasses provide fit_normalization, train_step, predict_into, _cast,
    _snapshot / _restore (copies of the trainable FP32 parameters) and the
    `status` word of their contractions."""

    frozen = False

    @staticmethod
    def _finite_rows(data: TrainingSet, n):
        """Indices (host) of the first n stored pairs whose position and
        gradient (and misfit, when kept) are finite: trajectories that
        diverged record non-finite values, which must not reach the
        normalisation or the loss."""
        import torch

        ok = torch.isfinite(data.q[:n]).all(dim=1) & torch.isfinite(data.g[:n]).all(dim=1)
        if data.with_values:
            ok &= torch.isfinite(data.x[:n])
        return _np.flatnonzero(ok.cpu().numpy())

    def train(self, data: TrainingSet, steps=2000, batch=256, lr=1e-3, seed=0, lr_decay=True, stream=None, rows=None,
              recent=None):
        """Fit the network with Adam on the first `rows` pairs of data (all by
        default; pairs with non-finite entries are skipped); with `recent`,
        half of every minibatch comes from the last `recent` usable pairs.
        Returns the loss history (host)."""
        rng = _np.random.default_rng(seed)
        n = data.count if rows is None else min(int(rows), data.count)
        usable = self._finite_rows(data, n)
        assert len(usable) >= batch, "not enough (finite) training pairs"
        tail = usable[-int(recent):] if recent else None
        history = []
        for s in range(steps):
            rate = lr * (0.5 * (1 + _np.cos(_np.pi * s / steps)) if lr_decay else 1.0)
            if tail is not None:
                h = batch // 2
                idx = _np.concatenate([usable[rng.integers(0, len(usable), size=batch - h)],
                                       tail[rng.integers(0, len(tail), size=h)]])
            else:
                idx = usable[rng.integers(0, len(usable), size=batch)]
            loss = self.train_step(data, idx, lr=float(rate), stream=stream)
            if s % 50 == 0 or s == steps - 1:
                history.append((s, float(loss[0].item())))
        self.check_status()
        return history

    def refresh(self, data: TrainingSet, steps=300, lr=2e-4, recent=640, seed=0, stream=None):
        """Continue training on pairs appended since the fit (for example
        exact gradients at the chains' current positions) with the fit's
        normalisation kept, then freeze again.  Used between blocks of
        surrogate-driven proposals: every block runs with a fixed network,
        so each block's kernel leaves the exact posterior invariant."""
        import contextlib

        import torch

        if stream is not None:
            stream.synchronize()  # the appended pairs were written on the sampler's stream; host reads follow
        self.frozen = False
        self._extend_targets(data)
        # every launch and copy of the training (index uploads included) on
        # the one stream, ordered after the sampler's work
        with torch.cuda.stream(stream) if stream is not None else contextlib.nullcontext():
            self.train(data, steps=steps, lr=lr, seed=seed, lr_decay=False, recent=recent)
        return self.freeze()

    def _extend_targets(self, data: TrainingSet):
        """Per-pair targets that depend on the stored pairs (none here)."""

    def fit(self, data: TrainingSet, steps=3000, batch=256, lr=1e-3, holdout_fraction=0.1, check_every=200,
            seed=0, stream=None):
        """Train with early stopping: a random `holdout_fraction` of the stored
        pairs is held out, and every `check_every` steps its relative error
        is measured; the weights with the lowest one are kept.  Returns a
        dict with the loss history, the held-out errors (step 0 is the
        least-squares linear start) and the best step.  Pairs with non-finite
        entries are left out of both sets."""
        import torch

        usable = self._finite_rows(data, data.count)
        n = len(usable)
        rng = _np.random.default_rng(seed)
        perm = usable[rng.permutation(n)]
        n_hold = max(1, int(round(holdout_fraction * n)))
        held = torch.from_numpy(_np.sort(perm[:n_hold])).to(self.device)
        train_rows = _np.sort(perm[n_hold:])
        assert len(train_rows) >= batch, "not enough training pairs"
        self.fit_normalization(data, rows=train_rows)
        value_err = getattr(self, "value_error", None)

        def score():
            # model selection: the held-out value error when values are
            # matched (what the acceptance sees), else the gradient error
            e = self.relative_error(data, held, stream=stream)
            ve = value_err(data, held, stream=stream) if value_err is not None else None
            return e, ve, (ve if ve is not None else e)

        err0, verr0, s0 = score()
        best = (s0, 0, self._snapshot())
        errors, verrors = [(0, err0)], [(0, verr0)]
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
            e, ve, sc = score()
            errors.append((done, e))
            verrors.append((done, ve))
            if sc < best[0]:
                best = (sc, done, self._snapshot())
        self.check_status()
        self._restore(best[2])
        self._cast(_dev.stream_handle(stream))
        torch.cuda.synchronize(self.device)
        at_best = dict(errors)[best[1]]
        return {"history": history, "heldout": errors, "heldout_value": verrors, "best_step": best[1],
                "best_heldout": at_best, "best_heldout_value": dict(verrors)[best[1]],
                "train_pairs": len(train_rows), "heldout_pairs": n_hold, "skipped_pairs": data.count - n}

    def freeze(self):
        self.frozen = True
        return self

    # ---- checkpoints -----------------------------------------------------------
    def _state_tensors(self):
        """name -> FP32 device tensor of everything training and prediction
        read (master weights, Adam moments, normalisation); the BF16 copies
        are derived from these."""
        raise NotImplementedError

    def state_arrays(self):
        """Host copies of the surrogate's state: continuing training or
        sampling from `load_state_arrays` of these is bit for bit the same as
        continuing this object."""
        out = {k: v.detach().cpu().numpy().copy() for k, v in self._state_tensors().items()}
        out["steps"] = _np.array(self.steps, _np.int64)
        out["frozen"] = _np.array(bool(self.frozen))
        out["kind"] = _np.array(type(self).__name__)
        return out

    def load_state_arrays(self, arrays):
        import torch

        kind = str(arrays["kind"])
        if kind != type(self).__name__:
            raise ValueError(f"checkpoint holds a {kind}, not a {type(self).__name__}")
        for k, t in self._state_tensors().items():
            a = _np.asarray(arrays[k])
            if a.shape != tuple(t.shape):
                raise ValueError(f"checkpoint entry {k} has shape {a.shape}, the surrogate {tuple(t.shape)}")
            t.copy_(torch.from_numpy(a).to(t.device, t.dtype))
        self.steps = int(arrays["steps"])
        self.frozen = bool(arrays["frozen"])
        self._recast(_dev.stream_handle())
        torch.cuda.synchronize(self.device)
        return self

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


class MLPSurrogate(_Surrogate):
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

    # ---- inference for the sampler -----------------------------------------
    def predict_into(self, q, g, stream):
        """g [d][C] = surrogate gradient at the chain positions q [d][C]."""
        C = q.shape[1]
        b = self._buffers(C, False)
        _lib.call("hmc_mlp_input", self.d, C, q.data_ptr(), self.mu_q.data_ptr(), self.inv_q.data_ptr(),
                  b["X"].data_ptr(), b["A2"].shape[1], stream)
        self._forward(b, C, stream, g_state=g)

    def _state_tensors(self):
        t = {}
        for l in range(3):
            for name, lst in (("W", self.W), ("b", self.b), ("mW", self.mW), ("vW", self.vW), ("mb", self.mb),
                              ("vb", self.vb)):
                t[f"{name}{l}"] = lst[l]
        for name in ("mu_q", "inv_q", "mu_g", "sig_g", "inv_g"):
            t[name] = getattr(self, name)
        return t

    def _recast(self, stream):
        self._cast(stream)

    def _snapshot(self):
        return [w.clone() for w in self.W] + [b.clone() for b in self.b]

    def _restore(self, snap):
        for l in range(3):
            self.W[l].copy_(snap[l])
            self.b[l].copy_(snap[3 + l])



def quadratic_fit(x, y, ridge=1e-3):
    """Gradient of the quadratic x^T A x / 2 + beta . x closest to the pairs
    (x_k, y_k) (rows of x, y): the ridge least-squares affine map
    y ~ x A^T + beta (penalty ridge * n on A, none on beta), with A then
    replaced by its symmetric part, the Hessian of a potential.  Host FP64."""
    n, d = x.shape
    x1 = _np.c_[x, _np.ones((n, 1))]
    reg = ridge * n * _np.eye(d + 1)
    reg[-1, -1] = 0.0
    sol = _np.linalg.solve(x1.T @ x1 + reg, x1.T @ y)
    A = sol[:d].T
    return 0.5 * (A + A.T), sol[d]


class PotentialSurrogate(_Surrogate):
    """Scalar-potential surrogate: f(x) = w3 . GELU(W2 GELU(W1 x + b1) + b2)
    + x^T A x / 2 + beta . x of x = (q - mu_q) / s_q, with the leapfrog driven
    by grad_q f = grad_x f / s_q.

    A network that outputs a gradient directly defines a force field with a
    curl: along a trajectory it pumps energy in or out, and the acceptance of
    the exact test decays with the trajectory length.  The gradient of a
    scalar is curl-free, so the surrogate dynamics conserve the surrogate
    Hamiltonian up to the integrator's error, and only the potential's own
    error enters the acceptance.  A and beta are the symmetrised ridge fit of
    the training gradients (the quadratic part of U); the network learns the
    rest by matching its gradient to the exact gradients
    (loss 0.5 mean |(grad_q f - g) / sigma_g|^2), which the project's kernels
    differentiate with respect to the weights by double backpropagation
    (csrc/potential.cu).  Same interface as MLPSurrogate."""

    def __init__(self, dimensions, hidden=(512, 512), seed=0, device=None):
        import torch

        self.device = device or _dev.require_cuda()
        d, h1, h2 = int(dimensions), int(hidden[0]), int(hidden[1])
        assert h1 % 16 == 0 and h2 % 16 == 0, "hidden widths must be multiples of 16"
        self.d = d
        self.sizes = [d, h1, h2]
        self.kg = h1 + d  # the output contraction reads [delta1 | x]
        rng = _np.random.default_rng(seed)
        f32 = dict(dtype=torch.float32, device=self.device)
        bf = dict(dtype=torch.bfloat16, device=self.device)

        def uniform(bound, shape):
            return torch.from_numpy(rng.uniform(-bound, bound, size=shape)).to(**f32).contiguous()

        # uniform +-1/sqrt(fan_in); the output weights 10x smaller, so training
        # starts from the quadratic fit
        self.params = {
            "W1": uniform(d**-0.5, (h1, d)), "b1": uniform(d**-0.5, (h1,)),
            "W2": uniform(h1**-0.5, (h2, h1)), "b2": uniform(h1**-0.5, (h2,)),
            "w3": uniform(0.1 * h2**-0.5, (h2,)),
        }
        self.grads = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.m1 = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.m2 = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.A = torch.zeros((d, d), **f32)
        self.beta = torch.zeros(d, **f32)
        self.mu_q = torch.zeros(d, **f32)
        self.inv_q = torch.ones(d, **f32)
        self.mu_g = torch.zeros(d, **f32)
        self.sig_g = torch.ones(d, **f32)
        self.inv_g = torch.ones(d, **f32)
        self.scale = torch.ones(d, **f32)  # 1 / (s_q sigma_g): grad_x f -> normalised gradient
        self.bias_out = torch.zeros(d, **f32)  # scale * beta - mu_g / sigma_g
        self.zero_h1 = torch.zeros(h1, **f32)
        self.zero_h2 = torch.zeros(h2, **f32)
        self.W1_16 = torch.zeros((h1, _pad(d)), **bf)
        self.W1t_16 = torch.zeros((d, _pad(h1)), **bf)
        self.W2_16 = torch.zeros((h2, _pad(h1)), **bf)
        self.W2t_16 = torch.zeros((h1, _pad(h2)), **bf)
        self.Wg = torch.zeros((d, _pad(self.kg)), **bf)  # [scale W1^T | scale A]
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.loss_buf = torch.zeros(1025, dtype=torch.float64, device=self.device)
        self.value_loss = torch.zeros(1, dtype=torch.float64, device=self.device)
        # value matching (off unless value_weight > 0 and the training set keeps misfits)
        self.value_weight = 0.0
        self._vt = None  # per stored pair: U minus the quadratic part (FP64, device)
        self._vt_w = 0.0
        self.steps = 0
        self._bufs = {}
        h = _dev.stream_handle()
        self._cast(h)
        self._cast_quadratic(h)
        self.frozen = False

    # ---- buffers and weights -------------------------------------------------
    def _buffers(self, B, training):
        import torch

        key = (int(B), bool(training))
        if key in self._bufs:
            return self._bufs[key]
        bf, f32 = torch.bfloat16, torch.float32
        d, h1, h2 = self.sizes
        pB = _pad(B)
        z = lambda shape, dt: torch.zeros(shape, dtype=dt, device=self.device)  # noqa: E731
        Ag = z((B, _pad(self.kg)), bf)
        b = {
            "Ag": Ag, "X": Ag[:, h1:],
            "Z1": z((B, h1), f32), "A1": z((B, _pad(h1)), bf), "A1t": z((h1, pB), bf),
            "Z2": z((B, h2), f32), "A2": z((B, _pad(h2)), bf), "A2t": z((h2, pB), bf),
            "D2": z((B, _pad(h2)), bf), "U1": z((B, h1), f32),
        }
        if training:
            b.update({
                "idx": z((B,), torch.int32), "Xt": z((d, pB), bf), "T": z((B, d), f32), "Y": z((B, d), f32),
                "D2t": z((h2, pB), bf), "D1t": z((h1, pB), bf),
                "E": z((B, _pad(d)), bf), "Et": z((d, pB), bf),
                "DB1": z((B, h1), f32), "UB1": z((B, _pad(h1)), bf), "UB1t": z((h1, pB), bf),
                "ZB1p": z((B, h1), f32), "DB2": z((B, h2), f32),
                "ZB2": z((B, _pad(h2)), bf), "ZB2t": z((h2, pB), bf),
                "AB1": z((B, h1), f32), "ZB1": z((B, _pad(h1)), bf), "ZB1t": z((h1, pB), bf),
                "dv": z((B,), f32), "S2t": z((h2, pB), bf), "S1t": z((h1, pB), bf),
            })
        self._bufs[key] = b
        return b

    def _cast(self, stream):
        d, h1, h2 = self.sizes
        P = self.params
        _lib.call("hmc_mlp_cast", h1, d, P["W1"].data_ptr(), self.W1_16.data_ptr(), _pad(d), self.W1t_16.data_ptr(),
                  _pad(h1), stream)
        _lib.call("hmc_mlp_cast", h2, h1, P["W2"].data_ptr(), self.W2_16.data_ptr(), _pad(h1),
                  self.W2t_16.data_ptr(), _pad(h2), stream)
        _lib.call("hmc_pot_scaled_cast", d, h1, P["W1"].data_ptr(), d, 1, self.scale.data_ptr(), self.Wg.data_ptr(),
                  self.Wg.shape[1], 0, stream)

    def _cast_quadratic(self, stream):
        d, h1, _ = self.sizes
        _lib.call("hmc_pot_scaled_cast", d, d, self.A.data_ptr(), d, 0, self.scale.data_ptr(), self.Wg.data_ptr(),
                  self.Wg.shape[1], h1, stream)

    def _out(self, **kw):
        o = _lib.HmcMlpOut()
        for k, v in kw.items():
            setattr(o, k, v.data_ptr() if hasattr(v, "data_ptr") else v)
        return o

    def _mm(self, mode, M, N, K, x, ldx, w, bias, out, stream):
        import ctypes

        _lib.call("hmc_tc_mlp", mode, M, N, K, x.data_ptr(), ldx, w.data_ptr(), w.shape[1],
                  bias.data_ptr() if bias is not None else None, ctypes.byref(out), self.status.data_ptr(), stream)

    def _ew(self, mode, B, n, stream, z, out_bf, out_t=None, inp=None, aux=None, vec=None, out_f=None):
        _lib.call("hmc_pot_elementwise", mode, B, n, _dev.ptr(inp), inp.shape[1] if inp is not None else 0,
                  z.data_ptr(), z.shape[1], _dev.ptr(aux), aux.shape[1] if aux is not None else 0, _dev.ptr(vec),
                  out_bf.data_ptr(), out_bf.stride(0), _dev.ptr(out_t), out_t.shape[1] if out_t is not None else 0,
                  _dev.ptr(out_f), out_f.shape[1] if out_f is not None else 0, stream)

    def _gradient_pass(self, b, B, stream, training, g_state=None):
        """grad_x f of the rows of b["X"], normalised (y = scale grad_x f +
        bias_out) into b["Y"], or as grad_q f into g_state [d][B]."""
        d, h1, h2 = self.sizes
        P = self.params
        pB = _pad(B)
        ldg = b["Ag"].shape[1]
        o = self._out(z=b["Z1"], ldz=h1, act=b["A1"], ld_act=_pad(h1), act_t=b["A1t"], ld_act_t=pB)
        self._mm(_lib.HMC_MLP_HIDDEN, B, h1, d, b["X"], ldg, self.W1_16, P["b1"], o, stream)
        o = self._out(z=b["Z2"], ldz=h2, act=b["A2"], ld_act=_pad(h2), act_t=b["A2t"], ld_act_t=pB)
        self._mm(_lib.HMC_MLP_HIDDEN, B, h2, h1, b["A1"], _pad(h1), self.W2_16, P["b2"], o, stream)
        self._ew(_lib.HMC_POT_DELTA2, B, h2, stream, b["Z2"], b["D2"], b.get("D2t") if training else None,
                 vec=P["w3"])
        self._mm(_lib.HMC_MLP_OUT, B, h1, h2, b["D2"], _pad(h2), self.W2t_16, self.zero_h1,
                 self._out(y=b["U1"], ldy=h1), stream)
        self._ew(_lib.HMC_POT_DELTA1, B, h1, stream, b["Z1"], b["Ag"], b.get("D1t") if training else None,
                 inp=b["U1"])
        if g_state is None:
            o = self._out(y=b["Y"], ldy=d)
        else:
            o = self._out(g_state=g_state, out_scale=self.sig_g, out_shift=self.mu_g)
        self._mm(_lib.HMC_MLP_OUT, B, d, self.kg, b["Ag"], ldg, self.Wg, self.bias_out, o, stream)

    # ---- normalisation and the quadratic part --------------------------------
    def fit_normalization(self, data: TrainingSet, rows=None):
        """Per-coordinate scales and the quadratic part A, beta: the ridge
        least-squares fit grad_x U ~ A x + beta on the stored pairs (or the
        given rows), symmetrised."""
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
        scale = 1.0 / (sq * sg)
        self.scale.copy_(scale.float())
        x = ((q - q.mean(dim=0)) / sq).cpu().numpy()
        y = (g * sq).cpu().numpy()  # grad_x U
        A, beta = quadratic_fit(x, y)
        self.A.copy_(torch.from_numpy(A).float())
        self.beta.copy_(torch.from_numpy(beta).float())
        self.bias_out.copy_((scale * self.beta.double() - g.mean(dim=0) / sg).float())
        h = _dev.stream_handle()
        self._cast(h)
        self._cast_quadratic(h)
        self._value_targets(data, rows, A, beta)
        torch.cuda.synchronize(self.device)

    def _value_targets(self, data: TrainingSet, rows, A, beta):
        """Value-matching targets of every stored pair: the exact misfit
        minus the quadratic part x^T A x / 2 + beta . x (the part the network
        does not learn), and the loss weight value_weight / var(targets)."""
        import torch

        self._vt = None
        self._quad_host = (A, beta)
        if not (self.value_weight > 0 and data.with_values):
            return
        n = data.count
        t = self._targets_host(data, 0, n)
        sel = _np.arange(n) if rows is None else _np.asarray(rows)
        sel = sel[_np.isfinite(t[sel])]
        var = float(_np.var(t[sel])) if sel.size > 1 else 1.0
        self._vt_w = float(self.value_weight / max(var, 1e-300))
        self._vt = torch.from_numpy(_np.where(_np.isfinite(t), t, 0.0)).to(self.device)

    def _targets_host(self, data: TrainingSet, start, stop):
        """Exact misfit minus the quadratic part at stored pairs [start, stop)."""
        A, beta = self._quad_host
        q = data.q[start:stop].double().cpu().numpy()
        x = (q - self.mu_q.double().cpu().numpy()) * self.inv_q.double().cpu().numpy()
        U = data.x[start:stop].cpu().numpy()
        return U - (0.5 * _np.einsum("bi,ij,bj->b", x, A, x) + x @ beta)

    def _extend_targets(self, data: TrainingSet):
        """Value targets of pairs stored after the fit (the quadratic part and
        the normalisation stay those of the fit)."""
        import torch

        if self._vt is None or data.count <= self._vt.numel():
            return
        t = self._targets_host(data, self._vt.numel(), data.count)
        t = torch.from_numpy(_np.where(_np.isfinite(t), t, 0.0)).to(self.device)
        self._vt = torch.cat([self._vt, t])

    def value_error(self, data: TrainingSet, rows, stream=None):
        """Standard deviation over the given stored pairs (at most 1024) of
        f(q) - U(q) about its mean, in misfit units: the potential's error
        that enters the acceptance of a surrogate trajectory through the
        difference of its end points.  None when values are not matched."""
        import torch

        if self._vt is None:
            return None
        rows = _np.asarray(rows.cpu().numpy() if hasattr(rows, "cpu") else rows)[:1024]
        B = len(rows)
        q = data.q[torch.as_tensor(rows, device=self.device)].t().contiguous()
        g = torch.empty_like(q)
        h = _dev.stream_handle(stream)
        self.predict_into(q, g, h)
        b = self._bufs[(B, False)]
        idx = torch.as_tensor(rows.astype(_np.int32), device=self.device)
        dv = torch.empty(B, dtype=torch.float32, device=self.device)
        _lib.call("hmc_pot_value_residual", B, self.sizes[2], b["A2"].data_ptr(), b["A2"].shape[1],
                  self.params["w3"].data_ptr(), self._vt.data_ptr(), idx.data_ptr(), 1.0, dv.data_ptr(),
                  self.value_loss.data_ptr(), h)
        return float(_np.sqrt(2.0 * self.value_loss.item()))

    # ---- training --------------------------------------------------------------
    def train_step(self, data: TrainingSet, idx_host, lr=1e-3, stream=None, beta1=0.9, beta2=0.999, eps=1e-8):
        """One Adam step of gradient matching on the minibatch rows idx_host;
        returns the device loss buffer (loss_buf[0])."""
        import torch

        assert not self.frozen, "the surrogate is frozen"
        h = _dev.stream_handle(stream)
        B = len(idx_host)
        b = self._buffers(B, True)
        d, h1, h2 = self.sizes
        P, G = self.params, self.grads
        pB = _pad(B)
        b["idx"].copy_(torch.from_numpy(_np.asarray(idx_host, _np.int32)), non_blocking=False)
        _lib.call("hmc_mlp_gather", B, d, b["idx"].data_ptr(), data.q.data_ptr(), data.g.data_ptr(),
                  self.mu_q.data_ptr(), self.inv_q.data_ptr(), self.mu_g.data_ptr(), self.inv_g.data_ptr(),
                  b["X"].data_ptr(), b["Ag"].shape[1], b["Xt"].data_ptr(), pB, b["T"].data_ptr(), d, h)
        self._gradient_pass(b, B, h, True)
        _lib.call("hmc_pot_loss", B, d, b["Y"].data_ptr(), d, b["T"].data_ptr(), d, self.scale.data_ptr(),
                  b["E"].data_ptr(), _pad(d), b["Et"].data_ptr(), pB, self.loss_buf.data_ptr(), h)
        # dW1 = delta1^T e; dbar1 = e W1^T -> ubar1, zbar1 (partial)
        self._wgrad(d, h1, B, b["Et"], b["D1t"], G["W1"], 0, h)
        self._mm(_lib.HMC_MLP_OUT, B, h1, d, b["E"], _pad(d), self.W1_16, self.zero_h1,
                 self._out(y=b["DB1"], ldy=h1), h)
        self._ew(_lib.HMC_POT_DBAR1, B, h1, h, b["Z1"], b["UB1"], b["UB1t"], inp=b["DB1"], aux=b["U1"],
                 out_f=b["ZB1p"])
        # dW2 = delta2^T ubar1; dbar2 = ubar1 W2^T -> dw3, zbar2
        self._wgrad(h1, h2, B, b["UB1t"], b["D2t"], G["W2"], 0, h)
        self._mm(_lib.HMC_MLP_OUT, B, h2, h1, b["UB1"], _pad(h1), self.W2_16, self.zero_h2,
                 self._out(y=b["DB2"], ldy=h2), h)
        _lib.call("hmc_pot_w3_grad", B, h2, b["DB2"].data_ptr(), h2, b["Z2"].data_ptr(), h2, G["w3"].data_ptr(), h)
        self._ew(_lib.HMC_POT_DBAR2, B, h2, h, b["Z2"], b["ZB2"], b["ZB2t"], inp=b["DB2"], vec=P["w3"])
        # abar1 = zbar2 W2 -> zbar1; the forward pass's weight and bias gradients
        self._mm(_lib.HMC_MLP_OUT, B, h1, h2, b["ZB2"], _pad(h2), self.W2t_16, self.zero_h1,
                 self._out(y=b["AB1"], ldy=h1), h)
        self._ew(_lib.HMC_POT_ZBAR1, B, h1, h, b["Z1"], b["ZB1"], b["ZB1t"], inp=b["AB1"], aux=b["ZB1p"])
        self._wgrad(h1, h2, B, b["A1t"], b["ZB2t"], G["W2"], 1, h)
        _lib.call("hmc_mlp_bias_grad", h2, B, b["ZB2t"].data_ptr(), pB, G["b2"].data_ptr(), h)
        self._wgrad(d, h1, B, b["Xt"], b["ZB1t"], G["W1"], 1, h)
        _lib.call("hmc_mlp_bias_grad", h1, B, b["ZB1t"].data_ptr(), pB, G["b1"].data_ptr(), h)
        if self._vt is not None and self._vt_w > 0:
            self._value_step(b, B, h)
        self.steps += 1
        for k in P:
            _lib.call("hmc_mlp_adam", P[k].numel(), P[k].data_ptr(), G[k].data_ptr(), self.m1[k].data_ptr(),
                      self.m2[k].data_ptr(), lr, beta1, beta2, eps, self.steps, h)
        self._cast(h)
        return self.loss_buf

    def _wgrad(self, n_in, n_out, B, act_t, delta_t, g, accumulate, stream):
        """g [n_out][n_in] (+)= sum_b delta[b][out] act[b][in] (K = batch)."""
        import ctypes

        o = self._out(g=g, accumulate=int(accumulate))
        _lib.call("hmc_tc_mlp", _lib.HMC_MLP_WGRAD, n_in, n_out, B, act_t.data_ptr(), act_t.shape[1],
                  delta_t.data_ptr(), delta_t.shape[1], None, ctypes.byref(o), self.status.data_ptr(), stream)

    def _value_step(self, b, B, h):
        """Add the value-matching loss's weight gradients to self.grads (the
        forward and gradient passes of this step left a2, delta2, delta1,
        a1 and x in the buffers; see csrc/potential.cu)."""
        d, h1, h2 = self.sizes
        P, G = self.params, self.grads
        pB = _pad(B)
        _lib.call("hmc_pot_value_residual", B, h2, b["A2"].data_ptr(), b["A2"].shape[1], P["w3"].data_ptr(),
                  self._vt.data_ptr(), b["idx"].data_ptr(), float(self._vt_w), b["dv"].data_ptr(),
                  self.value_loss.data_ptr(), h)
        # z2 = W2 a1 + b2: dz2 = dv delta2
        _lib.call("hmc_pot_scale_columns", h2, B, b["D2t"].data_ptr(), pB, b["dv"].data_ptr(), b["S2t"].data_ptr(),
                  pB, h)
        self._wgrad(h1, h2, B, b["A1t"], b["S2t"], G["W2"], 1, h)
        _lib.call("hmc_pot_weighted_colsum", B, h2, b["D2"].data_ptr(), b["D2"].shape[1], b["dv"].data_ptr(),
                  G["b2"].data_ptr(), h)
        # z1 = W1 x + b1: dz1 = dv delta1 (delta1 sits in the first h1 columns of Ag)
        _lib.call("hmc_pot_scale_columns", h1, B, b["D1t"].data_ptr(), pB, b["dv"].data_ptr(), b["S1t"].data_ptr(),
                  pB, h)
        self._wgrad(d, h1, B, b["Xt"], b["S1t"], G["W1"], 1, h)
        _lib.call("hmc_pot_weighted_colsum", B, h1, b["Ag"].data_ptr(), b["Ag"].shape[1], b["dv"].data_ptr(),
                  G["b1"].data_ptr(), h)
        # v = w3 . a2
        _lib.call("hmc_pot_weighted_colsum", B, h2, b["A2"].data_ptr(), b["A2"].shape[1], b["dv"].data_ptr(),
                  G["w3"].data_ptr(), h)

    def _state_tensors(self):
        t = {}
        for k in self.params:
            t[k] = self.params[k]
            t["m1_" + k] = self.m1[k]
            t["m2_" + k] = self.m2[k]
        for name in ("A", "beta", "mu_q", "inv_q", "mu_g", "sig_g", "inv_g", "scale", "bias_out"):
            t[name] = getattr(self, name)
        return t

    def _recast(self, stream):
        self._cast(stream)
        self._cast_quadratic(stream)

    def _snapshot(self):
        return {k: v.clone() for k, v in self.params.items()}

    def _restore(self, snap):
        for k, v in snap.items():
            self.params[k].copy_(v)

    # ---- inference for the sampler ---------------------------------------------
    def predict_into(self, q, g, stream):
        """g [d][C] = grad_q f at the chain positions q [d][C]."""
        C = q.shape[1]
        b = self._buffers(C, False)
        _lib.call("hmc_mlp_input", self.d, C, q.data_ptr(), self.mu_q.data_ptr(), self.inv_q.data_ptr(),
                  b["X"].data_ptr(), b["Ag"].shape[1], stream)
        self._gradient_pass(b, C, stream, False, g_state=g)
