"""Batched Hamiltonian Monte Carlo on one GPU.

`HMC(seed).sample(...)` keeps the reference signature (larsgeb/hmclab,
`hmclab/Samplers.py:1180-1311`) and semantics — position-Verlet leapfrog
(`:1524-1584`), 3-/4-stage integrators (`:1586-1726`), bound reflection after
every drift, FP64 Metropolis accept `exp(H0 - H1) > u` (`:1471-1492`),
optional Robbins-Monro step adaptation (`:1494-1522`), thinned samples
(`:675-678`), `max_time`, interrupts — and adds batched keyword arguments:

  chains        number of independent chains advanced together (default 1)
  dtype         'float64' (default for one chain) or 'float32' (default for
                batches): arithmetic type of positions, momenta, gradients;
                Hamiltonian sums and the accept test are always FP64
  rng_streams   None: counter-based Philox draws on the device (production);
                "numpy": replay `numpy.random.default_rng(seed + c)` per chain
                in the reference's draw order (reproduces the reference's
                chain for chains=1); or an explicit tuple (z, f, u) of arrays
                shaped [P][d][C], [P][C], [P][C]
  graph         capture each block of proposals in a CUDA graph (default True;
                targets whose `graph_safe` is False, e.g. the elastic FWI
                misfit with its own per-shot graphs, run uncaptured)
  keep_samples  keep every thinned sample on the device (`samples_device`)
  surrogate     a frozen `surrogate.PotentialSurrogate` or
                `surrogate.MLPSurrogate`: it supplies every gradient
                of the leapfrog; the exact misfit at the trajectory end still
                decides acceptance, so the chain targets the exact posterior
  training_set  a `surrogate.TrainingSet` that receives every exact
                (position, gradient) pair the trajectories evaluate, until it
                is full (burn-in data for the surrogate; runs uncaptured)
  temperatures  one temperature per chain: chain c targets
                exp(-misfit / T_c) (the tempered posteriors that the
                reference runs as separate distributions in parallel tempering)
  persistent    None (default): small dense linear-Gaussian targets (d <= 128)
                run whole blocks of proposals in one persistent launch, one
                warp per chain; False forces one launch per leapfrog step
  exchange_interval
                after every proposal whose index is a multiple of this (the
                first one included, as in the reference), the chains are
                paired at random and each pair swaps its models with the
                replica-exchange acceptance of `Samplers.py:589-669` (on the
                device)
  exchange_streams
                parity mode for the exchanges: (schedule [E][2 (C // 2)],
                uniforms [E][C // 2]) replacing the pairing and accept draws
                of exchange row e = proposal index // exchange_interval
  refresh_interval
                with a surrogate and a training_set: after every this many
                proposals the exact gradient (and misfit) at every chain's
                current position is appended to the training set and the
                surrogate trains `refresh_steps` more Adam steps at
                `refresh_lr` (half of each minibatch from the newest pairs),
                then freezes again; each block between refreshes runs with a
                fixed network, so its kernel keeps the exact posterior

diagnostic_mode (reference `Samplers.py:449-460, 499-527, 759-764`) times
every phase of the proposals with CUDA events on the sampler's stream:
momentum draw and trajectory start, gradients, kicks and drifts (with the
bound reflection), end-point misfits, the accept test, sample output and
replica exchanges.  Timing needs the launches uncaptured, so this mode runs
without CUDA graphs and without the persistent kernel.  `get_diagnostics()`
returns the timers (`function.__name__`, `calls`, `time_spent` in seconds);
`finish()` prints the split like the reference does.

Each proposal is issued as: begin (momentum, K0, first drift) -> for every
kick: gradient of the target on the device, then kick+drift -> misfit at the
end point -> accept/record.  All of it runs on one CUDA stream; blocks of
proposals are captured once and replayed as CUDA graphs.  Dense FP32 targets
with d >= 64 fuse the gradient, kick and drift into one tensor-core launch
per leapfrog step; small dense linear-Gaussian targets (d <= 128) run whole
blocks of proposals in one persistent launch (`run_together` advances several
such targets of different dimensions in the same launch).
"""
import ctypes as _ct
import os as _os
import time as _time
from datetime import datetime as _datetime

import numpy as _numpy

from hmclab_gb300 import _device as _dev
from hmclab_gb300 import _lib
from hmclab_gb300.Distributions import _AbstractDistribution
from hmclab_gb300.MassMatrices import Unit as _Unit, _AbstractMassMatrix
from hmclab_gb300.Samples import Samples as _Samples

try:
    import torch as _torch
except ImportError:  # pragma: no cover
    _torch = None

class DeviceTimer:
    """Accumulated device time of one phase of the proposals: the GPU
    counterpart of the reference's AccumulatingTimer (Helpers/Timers.py:23-60),
    with the same `function.__name__`, `calls` and `time_spent` (seconds)."""

    class _Name:
        def __init__(self, name):
            self.__name__ = name

    def __init__(self, name):
        self.function = DeviceTimer._Name(name)
        self.calls = 0
        self.time_spent = 0.0
        self._pending = []

    def begin(self, stream):
        ev = _torch.cuda.Event(enable_timing=True)
        ev.record(stream)
        return ev

    def end(self, ev0, stream):
        ev1 = _torch.cuda.Event(enable_timing=True)
        ev1.record(stream)
        self._pending.append((ev0, ev1))
        self.calls += 1

    def add_host_seconds(self, seconds):
        self.time_spent += float(seconds)
        self.calls += 1

    def collect(self):
        """Fold the finished event pairs into time_spent (synchronises on them)."""
        for ev0, ev1 in self._pending:
            ev1.synchronize()
            self.time_spent += ev0.elapsed_time(ev1) / 1e3
        self._pending.clear()

    def print_statistics(self):
        print(f"Function: {self.function.__name__}")
        print(f"Calls: {self.calls}")
        print(f"Total time spent: {self.time_spent} seconds")

    def __str__(self):
        return f"Function: {self.function.__name__}, Calls: {self.calls}, Total time spent: {self.time_spent} seconds, "


class _Phase:
    """Context manager that times a phase when the sampler has timers."""

    __slots__ = ("timer", "stream", "ev")

    def __init__(self, timer, stream):
        self.timer, self.stream = timer, stream

    def __enter__(self):
        if self.timer is not None:
            self.ev = self.timer.begin(self.stream)
        return self

    def __exit__(self, *exc):
        if self.timer is not None:
            self.timer.end(self.ev, self.stream)
        return False


_PHASES = ("generate_momentum", "gradient", "integrator", "misfit", "_evaluate_acceptance", "samples.append",
           "exchange")

# Integrator coefficients (Samplers.py:1588-1592, 1666-1669).
_A1_3S, _B1_3S = 0.11888010966548, 0.29619504261126
_A1_4S, _A2_4S, _B1_4S = 0.071353913450279725904, 0.268548791161230105820, 0.191667800000000000000


def integrator_ops(integrator, amount_of_steps):
    """The integrator as a list of ('d', a) drifts and ('k', b) kicks, where a
    and b multiply the step size."""
    ops = []
    if integrator == "lf":
        ops.append(("d", 0.5))
        for _ in range(amount_of_steps - 1):
            ops += [("k", 1.0), ("d", 1.0)]
        ops += [("k", 1.0), ("d", 0.5)]
    elif integrator == "3s":
        a1, b1 = _A1_3S, _B1_3S
        a2, b2 = 0.5 - a1, 1.0 - 2.0 * b1
        for _ in range(amount_of_steps):
            ops += [("d", a1), ("k", b1), ("d", a2), ("k", b2), ("d", a2), ("k", b1), ("d", a1)]
    elif integrator == "4s":
        a1, a2, b1 = _A1_4S, _A2_4S, _B1_4S
        a3, b2 = 1.0 - 2.0 * a1 - 2.0 * a2, 0.5 - b1
        for _ in range(amount_of_steps):
            ops += [("d", a1), ("k", b1), ("d", a2), ("k", b2), ("d", a3), ("k", b2), ("d", a2), ("k", b1), ("d", a1)]
    else:
        raise ValueError(f"Unknown integrator used. Choices are: {list(HMC.integrators_full_names)}")
    return ops


def compile_schedule(ops):
    """(first_drift, [(needs_gradient, kick, drift), ...]) for the device."""
    assert ops[0][0] == "d"
    first = ops[0][1]
    steps = []
    i = 1
    while i < len(ops):
        kind, c = ops[i]
        if kind == "k":
            drift = ops[i + 1][1] if i + 1 < len(ops) and ops[i + 1][0] == "d" else 0.0
            steps.append((True, c, drift))
            i += 2 if drift != 0.0 else 1
        else:
            steps.append((False, 0.0, c))
            i += 1
    return first, steps


class HMC:
    """Hamiltonian Monte Carlo over many chains on one GPU."""

    name = "Hamiltonian Monte Carlo"
    integrators_full_names = {"lf": "leapfrog integrator", "3s": "three stage integrator", "4s": "four stage integrator"}
    available_integrators = integrators_full_names.keys()
    minimal_stepsize = 1e-18
    surrogate = None
    training_set = None
    _temperatures = None
    exchange_interval = None
    _exchange_streams = None
    refresh_interval = None
    beta = None
    use_persistent = None
    _persistent = None
    _timers = None
    diagnostic_mode = False
    _proposal_base = 0  # proposals done before a resumed run (its Philox counter origin)

    def __init__(self, seed: int = None):
        self.seed = seed
        self.rng = _numpy.random.default_rng(seed)
        self.philox_seed = (
            int(seed) & 0xFFFFFFFFFFFFFFFF if seed is not None else int.from_bytes(_os.urandom(8), "little")
        )
        self.current_proposal = 0
        self.accepted_proposals = 0
        self.samples_device = None
        self.timings = {}

    # ------------------------------------------------------------------
    def sample(
        self,
        samples_filename,
        distribution: _AbstractDistribution,
        stepsize=0.1,
        randomize_stepsize: bool = True,
        amount_of_steps: int = 10,
        mass_matrix: _AbstractMassMatrix = None,
        integrator: str = "lf",
        initial_model=None,
        proposals: int = 100,
        online_thinning: int = 1,
        diagnostic_mode: bool = False,
        overwrite_existing_file: bool = False,
        max_time: float = None,
        autotuning: bool = False,
        target_acceptance_rate: float = 0.65,
        learning_rate: float = 0.75,
        queue=None,
        disable_progressbar=False,
        chains: int = None,
        dtype=None,
        rng_streams=None,
        graph: bool = True,
        proposals_per_graph: int = None,
        keep_samples: bool = False,
        surrogate=None,
        training_set=None,
        temperatures=None,
        exchange_interval: int = None,
        persistent: bool = None,
        resume=None,
        exchange_streams=None,
        refresh_interval: int = None,
        refresh_steps: int = 300,
        refresh_lr: float = 2e-4,
    ):
        """Run `proposals` HMC proposals for every chain; returns self.

        `resume` (a path written by `checkpoint()`) continues earlier chains:
        positions, per-chain step sizes, chain count, dtype, Philox key and
        proposal count (and a passed surrogate's state) come from the
        checkpoint.

        Raises AssertionError / ValueError / TypeError / FileExistsError for
        invalid arguments like the reference."""
        self.disable_progressbar = disable_progressbar
        self.prepare(
            samples_filename, distribution, stepsize=stepsize, randomize_stepsize=randomize_stepsize,
            amount_of_steps=amount_of_steps, mass_matrix=mass_matrix, integrator=integrator,
            initial_model=initial_model, proposals=proposals, online_thinning=online_thinning,
            diagnostic_mode=diagnostic_mode, overwrite_existing_file=overwrite_existing_file, max_time=max_time,
            autotuning=autotuning, target_acceptance_rate=target_acceptance_rate, learning_rate=learning_rate,
            chains=chains, dtype=dtype, rng_streams=rng_streams, graph=graph, proposals_per_graph=proposals_per_graph,
            keep_samples=keep_samples, surrogate=surrogate, training_set=training_set, temperatures=temperatures,
            exchange_interval=exchange_interval, persistent=persistent, resume=resume,
            exchange_streams=exchange_streams, refresh_interval=refresh_interval, refresh_steps=refresh_steps,
            refresh_lr=refresh_lr,
        )
        self._run()
        return self

    # ------------------------------------------------------------------
    def _parse(self, samples_filename, distribution, stepsize, randomize_stepsize, amount_of_steps, mass_matrix,
               integrator, initial_model, proposals, online_thinning, diagnostic_mode, overwrite_existing_file,
               max_time, autotuning, target_acceptance_rate, learning_rate, chains, dtype, rng_streams, graph,
               proposals_per_graph, keep_samples):
        assert samples_filename is None or isinstance(samples_filename, (str, list, tuple)), (
            "First argument should be a string containing the path of the file to which to write samples."
        )
        assert issubclass(type(distribution), _AbstractDistribution), (
            "The passed target distribution should be a derived class of _AbstractDistribution."
        )
        assert type(distribution.dimensions) == int and distribution.dimensions > 0, (
            "The passed target distribution should have an integer dimension larger than zero."
        )
        self.distribution = distribution
        self.dimensions = distribution.dimensions
        assert type(proposals) == int and proposals > 0, (
            "The amount of proposal requested (`proposals`) should be an integer number larger than zero."
        )
        assert type(online_thinning) == int and online_thinning > 0, (
            "The amount of online thinning (`online_thinning`) should be an integer number larger than zero."
        )
        assert proposals % online_thinning == 0, (
            "The amount of proposals (`proposals`) needs to be a multiple of the online thinning "
            "(`online_thinning`) number, to prevent sample wastage."
        )
        self.proposals = proposals
        self.online_thinning = online_thinning
        self.proposals_after_thinning = proposals // online_thinning
        chains = 1 if chains is None else int(chains)
        assert chains > 0, "The number of chains should be a positive integer."
        self.chains = chains
        # default: FP64 for a single chain (the reference's arithmetic) unless
        # the target's kernels are FP32 only, FP32 for batches of chains
        single = getattr(distribution, "single_dtype", "float64")
        self.dtype = _dev.normalise_dtype(dtype) if dtype is not None else (single if chains == 1 else "float32")
        # step size: scalar or one per chain
        eps = _numpy.asarray(stepsize, dtype=_numpy.float64).reshape(-1)
        assert eps.size in (1, chains), "stepsize must be a scalar or one value per chain"
        assert _numpy.all(eps > 0.0), "Stepsize should be a float larger than zero."
        self.stepsize = float(eps[0]) if eps.size == 1 else eps.copy()
        self._eps0 = _numpy.broadcast_to(eps, (chains,)).astype(_numpy.float64).copy()
        self.randomize_stepsize = bool(randomize_stepsize)
        assert type(amount_of_steps) == int, (
            "The amount of steps (amount_of_steps) the HMC integrator should make should be an integer."
        )
        assert amount_of_steps > 0, (
            "The amount of steps (amount_of_steps) the HMC integrator should make should be larger than zero."
        )
        self.amount_of_steps = amount_of_steps
        if mass_matrix is None:
            mass_matrix = _Unit(self.dimensions)
        if mass_matrix.kind is None:
            raise NotImplementedError(
                f"{type(mass_matrix).__name__} updates the mass inside the trajectory, which the batched device "
                "sampler does not do (it would make the chain inexact); learn it on the host and pass "
                "freeze(cast=True), a Full mass matrix")
        mass_matrix.rng = self.rng
        assert isinstance(mass_matrix, _AbstractMassMatrix), (
            "The passed mass matrix (mass_matrix) should be a class derived from _AbstractMassMatrix."
        )
        assert mass_matrix.dimensions == self.dimensions, (
            "The passed mass matrix (mass_matrix) should have dimensions equal to the target distribution. "
            f"Passed: {mass_matrix.dimensions}, required: {self.dimensions}."
        )
        self.mass_matrix = mass_matrix
        self.integrator = str(integrator)
        if self.integrator not in self.available_integrators:
            raise ValueError(f"Unknown integrator used. Choices are: {self.available_integrators}")
        self.autotuning = bool(autotuning)
        if self.autotuning:
            assert 0.5 < learning_rate <= 1.0, (
                "The learning rate should be larger than 0.5 and smaller than or equal to 1.0, otherwise the "
                f"Markov chain does not converge. Chosen: {learning_rate}"
            )
        self.target_acceptance_rate = float(target_acceptance_rate)
        self.learning_rate = float(learning_rate)
        # initial model: (d,1) broadcast to every chain, or (d, C)
        if initial_model is None:
            q0 = _numpy.zeros((self.dimensions, chains))
        else:
            q0 = _numpy.array(initial_model, dtype=_numpy.float64)
            if q0.size == self.dimensions:
                q0 = _numpy.repeat(q0.reshape(self.dimensions, 1), chains, axis=1)
            assert q0.shape == (self.dimensions, chains), (
                "The initial model (`initial_model`) dimension is incompatible with the target distribution. "
                f"Supplied model shape: {q0.shape}. Required shape: {(self.dimensions, 1)} or "
                f"{(self.dimensions, chains)}"
            )
        self._q0 = q0
        if max_time is not None:
            max_time = float(max_time)
            assert max_time > 0.0, "The maximal runtime (`max_time`) should be a float larger than zero."
        self.max_time = max_time
        self.diagnostic_mode = bool(diagnostic_mode)
        self.overwrite_existing_file = overwrite_existing_file
        self.samples_filename = samples_filename
        self.rng_streams = rng_streams
        self.use_graph = bool(graph)
        self.keep_samples = bool(keep_samples)
        if proposals_per_graph is None:
            k = max(1, 32 // online_thinning) * online_thinning
            proposals_per_graph = min(k, proposals)
        assert proposals_per_graph % online_thinning == 0, "proposals_per_graph must be a multiple of online_thinning"
        self.proposals_per_graph = int(proposals_per_graph)
        self._schedule = compile_schedule(integrator_ops(self.integrator, self.amount_of_steps))

    # ------------------------------------------------------------------
    def _filenames(self):
        fn = self.samples_filename
        if fn is None:
            return None
        if isinstance(fn, (list, tuple)):
            assert len(fn) == self.chains, "one samples filename per chain is required"
            return list(fn)
        if self.chains == 1:
            return [fn]
        stem, ext = _os.path.splitext(fn)
        return [f"{stem}.chain{c}{ext or '.npy'}" for c in range(self.chains)]

    def _open_files(self):
        names = self._filenames()
        self._writers = None
        if names is None:
            return
        writers = []
        try:
            for n in names:
                writers.append(_Samples(n, mode="w", overwrite=self.overwrite_existing_file))
        except Exception:
            for w in writers:
                w.close()
            raise
        self._writers = writers
        for w in writers:
            w.write_attribute("stepsize", self.stepsize if self.chains == 1 else list(self._eps0))
            w.write_attribute("amount_of_steps", self.amount_of_steps)
            w.write_attribute("mass_matrix", self.mass_matrix.name)
            w.write_attribute("integrator", self.integrators_full_names[self.integrator])
            w.write_attribute("proposals", self.proposals)
            w.write_attribute("acceptance_rate", 0)
            w.write_attribute("online_thinning", self.online_thinning)
            w.write_attribute("start_time", _datetime.now().strftime("%d-%b-%Y (%H:%M:%S.%f)"))
            w.write_attribute("sampler", self.name)

    # ------------------------------------------------------------------
    def _setup_device(self):
        dev = _dev.require_cuda()
        d, C, dt = self.dimensions, self.chains, self.dtype
        self.device = dev
        self.stream = _torch.cuda.Stream(device=dev)
        E = lambda shape, dtype=dt: _dev.empty(shape, dtype, dev)  # noqa: E731
        Z = lambda shape, dtype=dt: _dev.zeros(shape, dtype, dev)  # noqa: E731
        self.q_cur = _dev.upload(self._q0, dt, dev)
        self.q = self.q_cur.clone()
        self.p = Z((d, C))
        self.g = Z((d, C))
        self.v = Z((d, C)) if self.mass_matrix.kind == _lib.HMC_MASS_FULL else None
        self.eps = _dev.upload(self._eps0, dt, dev)
        self.eps_local = Z((C,))
        self.x_cur = Z((C,), "float64")
        self.x_prop = Z((C,), "float64")
        self.k_cur = Z((C,), "float64")
        self.k_prop = Z((C,), "float64")
        self.accepted = _torch.zeros((C,), dtype=_torch.int64, device=dev)
        self.beta = None
        if self._temperatures is not None:
            self.beta = _torch.from_numpy(1.0 / self._temperatures).to(dev)
        if self.exchange_interval is not None:
            self._ex_pairs = _torch.zeros((C,), dtype=_torch.int32, device=dev)
            self._ex_u = _torch.zeros((C // 2,), dtype=_torch.float64, device=dev)
            self._ex_swapped = _torch.zeros((C // 2,), dtype=_torch.int32, device=dev)
            self._ex_total = _torch.zeros((1,), dtype=_torch.int64, device=dev)
        self.flags = _torch.zeros((C,), dtype=_torch.int32, device=dev)
        self.control = _torch.zeros((2,), dtype=_torch.int64, device=dev)
        self.control[0] = self._proposal_base  # a resumed run continues the Philox counter
        lo, hi = self.distribution.lower_bounds, self.distribution.upper_bounds
        self.lower = _dev.upload(lo[:, 0], dt, dev) if lo is not None else None
        self.upper = _dev.upload(hi[:, 0], dt, dev) if hi is not None else None
        mp = self.mass_matrix.device_params(dt)
        # ring of thinned samples
        k = self.proposals_per_graph
        slots = self.proposals_after_thinning if self.keep_samples else k // self.online_thinning
        self.ring_slots = slots
        self.ring_q = E((slots, d, C))
        self.ring_x = E((slots, C), "float64")
        if self.autotuning:
            self.rec_eps = Z((self._proposal_base + self.proposals, C), "float64")
            self.rec_acc = Z((self._proposal_base + self.proposals, C), "float64")
        else:
            self.rec_eps = self.rec_acc = None
        # injected streams
        self._stream_chunk = None
        self.stream_z = self.stream_f = self.stream_u = None
        if self.rng_streams is not None:
            self.stream_z = E((k, d, C))
            self.stream_f = E((k, C))
            self.stream_u = E((k, C), "float64")
            if isinstance(self.rng_streams, str):
                if self.rng_streams != "numpy":
                    raise ValueError("rng_streams must be None, 'numpy' or a (z, f, u) tuple")
                base = 0 if self.seed is None else int(self.seed)
                self._numpy_rngs = [_numpy.random.default_rng(base + c) for c in range(C)]
            else:
                z, f, u = self.rng_streams
                z = _numpy.asarray(z, _numpy.float64).reshape(-1, d, C)
                f = _numpy.asarray(f, _numpy.float64).reshape(-1, C)
                u = _numpy.asarray(u, _numpy.float64).reshape(-1, C)
                assert z.shape[0] >= self.proposals and u.shape[0] >= self.proposals, "streams too short"
                self._explicit_streams = (z, f, u)
        st = _lib.HmcChains()
        st.dtype = _dev.dtype_code(dt)
        st.mass_kind = self.mass_matrix.kind
        st.dims, st.chains = d, C
        for name in ("q_cur", "q", "p", "g", "v", "eps", "eps_local", "x_cur", "x_prop", "k_cur", "k_prop",
                     "accepted", "flags"):
            setattr(st, name, _dev.ptr(getattr(self, name)))
        st.proposal = self.control.data_ptr()
        st.mass_diag = _dev.ptr(mp.get("diag"))
        st.mass_inv_diag = _dev.ptr(mp.get("inv_diag"))
        st.mass_chol = _dev.ptr(mp.get("chol"))
        st.mass_inv = _dev.ptr(mp.get("inv"))
        st.lower, st.upper = _dev.ptr(self.lower), _dev.ptr(self.upper)
        st.seed = self.philox_seed
        st.randomize_stepsize = int(self.randomize_stepsize)
        st.autotune = int(self.autotuning)
        st.target_acceptance = self.target_acceptance_rate
        st.learning_rate = self.learning_rate
        st.minimal_stepsize = self.minimal_stepsize
        st.stream_z, st.stream_eps, st.stream_u = _dev.ptr(self.stream_z), _dev.ptr(self.stream_f), _dev.ptr(self.stream_u)
        st.stream_len = k if self.rng_streams is not None else 0
        st.ring_q, st.ring_x = self.ring_q.data_ptr(), self.ring_x.data_ptr()
        st.ring_slots, st.thinning = slots, self.online_thinning
        st.rec_stepsize, st.rec_acceptance = _dev.ptr(self.rec_eps), _dev.ptr(self.rec_acc)
        st.rec_len = self._proposal_base + self.proposals if self.autotuning else 0
        st.beta = _dev.ptr(self.beta)
        self._state = st
        self._state_ref = _ct.byref(st)
        # Initial misfit (reference asserts it is finite, Samplers.py:419-426).
        self.stream.wait_stream(_torch.cuda.current_stream(dev))
        h = self.stream.cuda_stream
        self.distribution._device_misfit(self.q_cur, self.x_cur, False, dt, h)
        if self.use_graph:
            # allocate every scratch buffer of the target before any capture
            self.distribution._device_gradient(self.q_cur, self.g, False, dt, h)
            self.distribution._device_misfit(self.q_cur, self.x_prop, False, dt, h)
        self.stream.synchronize()
        x0 = self.x_cur.cpu().numpy()
        assert not _numpy.any(_numpy.isnan(x0)), "Initial position in model space gives NaN probability"
        assert not _numpy.any(_numpy.isinf(x0)), "Initial position in model space gives inf/-inf probability"
        self.current_x = x0[0] if C == 1 else x0
        self._graph = None
        from hmclab_gb300._dense_tc import FusedDenseStep

        from hmclab_gb300._persistent import PersistentDense

        self._persistent = PersistentDense.applies(self)
        self._fused = (
            None if (self._persistent is not None or self.surrogate is not None or self.training_set is not None)
            else FusedDenseStep.applies(self)
        )
        if self.surrogate is not None:
            self.surrogate._buffers(C, False)  # allocate before any capture
        self._training_x = Z((C,), "float64") if self.training_set is not None else None

    # ------------------------------------------------------------------
    def _phase(self, name):
        timers = self._timers
        return _Phase(timers[name] if timers is not None else None, self.stream)

    def _issue_proposal(self, h):
        """Enqueue one proposal for every chain on stream handle h."""
        st, dist, dt = self._state_ref, self.distribution, self.dtype
        first, steps = self._schedule
        with self._phase("generate_momentum"):
            _lib.call("hmc_begin_trajectory", st, first, h)
        fused = self._fused
        if fused is not None:
            # gradient + prior + kick + drift in the tensor-core epilogue
            with self._phase("integrator"):
                fused.after_begin(h)
                for needs_grad, kick, drift in steps:
                    if needs_grad:
                        fused.kick_drift(kick, drift, h)
                    else:
                        fused.drift_only(drift, h)
            with self._phase("misfit"):
                fused.misfit(h)
            with self._phase("_evaluate_acceptance"):
                _lib.call("hmc_end_trajectory", st, h)
            return
        for needs_grad, kick, drift in steps:
            if needs_grad:
                with self._phase("gradient"):
                    if self.surrogate is not None:
                        self.surrogate.predict_into(self.q, self.g, h)
                    else:
                        dist._device_gradient(self.q, self.g, False, dt, h)
                        if self.training_set is not None:
                            tx = None
                            if self.training_set.with_values:
                                tx = self._training_x
                                dist._device_misfit_after_gradient(self.q, tx, False, dt, h)
                            self.training_set.record(self.q, self.g, h, tx)
            with self._phase("integrator"):
                _lib.call("hmc_kick_drift", st, kick, drift, h)
        with self._phase("misfit"):
            dist._device_misfit(self.q, self.x_prop, False, dt, h)
        with self._phase("_evaluate_acceptance"):
            _lib.call("hmc_end_trajectory", st, h)

    def _issue_block(self, n_props, h):
        for _ in range(n_props):
            self._issue_proposal(h)

    def _load_streams(self, n0, n):
        """Copy the injected random streams of proposals [n0, n0+n) to the device."""
        if self.rng_streams is None:
            return
        d, C = self.dimensions, self.chains
        if isinstance(self.rng_streams, str):
            z = _numpy.empty((n, d, C))
            f = _numpy.ones((n, C))
            u = _numpy.empty((n, C))
            for c, rng in enumerate(self._numpy_rngs):
                for j in range(n):
                    z[j, :, c] = rng.normal(size=(d, 1))[:, 0]
                    if self.randomize_stepsize:
                        f[j, c] = rng.uniform(0.5, 1.5)
                    u[j, c] = rng.uniform(0, 1)
        else:
            zz, ff, uu = self._explicit_streams
            z, f, u = zz[n0 : n0 + n], ff[n0 : n0 + n], uu[n0 : n0 + n]
        # the device reads proposal g's draws from slot g % slots (g counts
        # from the chains' first proposal), so a block that does not start on
        # a multiple of the slot count wraps around
        slots = self.stream_z.shape[0]
        s0 = (self._proposal_base + n0) % slots
        parts = [(0, s0, min(n, slots - s0))]
        if parts[0][2] < n:
            parts.append((parts[0][2], 0, n - parts[0][2]))
        with _torch.cuda.stream(self.stream):
            for j0, t0, m in parts:
                for dst, src in ((self.stream_z, z), (self.stream_f, f), (self.stream_u, u)):
                    dst[t0:t0 + m].copy_(_torch.from_numpy(_numpy.ascontiguousarray(src[j0:j0 + m])).to(dst.dtype),
                                         non_blocking=False)

    def _drain(self, n0, n):
        """Move the thinned samples of proposals [n0, n0+n) to the files."""
        if self._writers is None or self.keep_samples:
            return
        first, m = self._recorded(n0, n)
        if m == 0:
            return
        sel = self._ring_index(first, m)
        with _torch.cuda.stream(self.stream):
            q = self.ring_q[sel].to(_torch.float64).cpu().numpy()  # m, d, C
            x = self.ring_x[sel].cpu().numpy()  # m, C
        for c, w in enumerate(self._writers):
            w.append_columns(_numpy.vstack([q[:, :, c].T, x[None, :, c]]))

    # ---- lower-level driving API (used by sample() and by benchmarks) ------
    def prepare(self, samples_filename, distribution, **kwargs):
        """Validate arguments, allocate the device state and open the files
        without running any proposal.  Takes the keyword arguments of sample()."""
        defaults = dict(
            stepsize=0.1, randomize_stepsize=True, amount_of_steps=10, mass_matrix=None, integrator="lf",
            initial_model=None, proposals=100, online_thinning=1, diagnostic_mode=False, overwrite_existing_file=False,
            max_time=None, autotuning=False, target_acceptance_rate=0.65, learning_rate=0.75, chains=None,
            dtype=None, rng_streams=None, graph=True, proposals_per_graph=None, keep_samples=False,
            surrogate=None, training_set=None, temperatures=None, exchange_interval=None, persistent=None,
            resume=None, exchange_streams=None, refresh_interval=None, refresh_steps=300, refresh_lr=2e-4,
        )
        unknown = set(kwargs) - set(defaults) - {"queue", "disable_progressbar"}
        if unknown:
            raise TypeError(f"Unidentified argument(s) not applicable to sampler: {unknown}")
        defaults.update({k: v for k, v in kwargs.items() if k in defaults})
        a = defaults
        ck = None
        if a["resume"] is not None:
            ck = self._read_checkpoint(a["resume"], distribution, a)
        self._parse(
            samples_filename, distribution, a["stepsize"], a["randomize_stepsize"], a["amount_of_steps"],
            a["mass_matrix"], a["integrator"], a["initial_model"], a["proposals"], a["online_thinning"],
            a["diagnostic_mode"], a["overwrite_existing_file"], a["max_time"], a["autotuning"],
            a["target_acceptance_rate"], a["learning_rate"], a["chains"], a["dtype"], a["rng_streams"], a["graph"],
            a["proposals_per_graph"], a["keep_samples"],
        )
        if ck is not None:
            self.philox_seed = int(ck["philox_seed"])
            self._proposal_base = int(ck["proposals_done"])
            if a["surrogate"] is not None:
                keys = [k for k in ck if k.startswith("surrogate.")]
                if not keys:
                    raise ValueError("the checkpoint holds no surrogate state to resume the surrogate from")
                a["surrogate"].load_state_arrays({k[len("surrogate."):]: ck[k] for k in keys})
        self._parse_surrogate(a["surrogate"], a["training_set"], a["refresh_interval"], a["refresh_steps"],
                              a["refresh_lr"])
        self._parse_tempering(a["temperatures"], a["exchange_interval"], a["exchange_streams"])
        self.use_persistent = a["persistent"]
        self._timers = None
        if self.diagnostic_mode:
            # every phase is timed with events: no graph capture, no persistent kernel
            self.use_graph = False
            self.use_persistent = False
            self._timers = {name: DeviceTimer(name) for name in _PHASES}
        self._setup_device()
        self._open_files()
        self._done = 0
        self._t0 = _time.time()
        self._start_time = _datetime.now()
        self._launches0 = _lib.launch_count()
        return self

    # ---- checkpoint / resume ------------------------------------------------
    CHECKPOINT_FORMAT = "hmclab_gb300.checkpoint.v1"

    def checkpoint(self, path):
        """Write what continuing these chains needs to `path` (.npz): current
        positions, per-chain base step sizes (as adapted by autotuning), the
        Philox key, the number of proposals done, and the surrogate's weights,
        Adam moments and normalisation when a surrogate drives the sampler.
        `sample(..., resume=path)` continues from it: with the same target,
        mass matrix and settings the continued chains equal an uninterrupted
        run bit for bit (the reference saves no chain or random state,
        Samples.py:280-335, so it has no counterpart)."""
        from hmclab_gb300.Helpers.CustomExceptions import InvalidCaseError

        if getattr(self, "current_model", None) is None:
            raise InvalidCaseError("checkpoint() needs a finished run (sample() or finish())")
        arrays = {
            "format": _numpy.array(self.CHECKPOINT_FORMAT),
            "q": _numpy.asarray(self.current_model, _numpy.float64),
            "eps": self.eps.to(_torch.float64).cpu().numpy(),
            "proposals_done": _numpy.array(self._proposal_base + self.proposals_done, _numpy.int64),
            "philox_seed": _numpy.array(self.philox_seed, _numpy.uint64),
            "dimensions": _numpy.array(self.dimensions, _numpy.int64),
            "chains": _numpy.array(self.chains, _numpy.int64),
            "dtype": _numpy.array(self.dtype),
            "online_thinning": _numpy.array(self.online_thinning, _numpy.int64),
        }
        if self.surrogate is not None:
            for k, v in self.surrogate.state_arrays().items():
                arrays["surrogate." + k] = v
        with open(path, "wb") as f:
            _numpy.savez(f, **arrays)
        return path

    def _read_checkpoint(self, path, distribution, a):
        """Load a checkpoint and fill the sampler arguments it determines."""
        with _numpy.load(path, allow_pickle=False) as f:
            ck = {k: f[k] for k in f.files}
        if str(ck.get("format", "")) != self.CHECKPOINT_FORMAT:
            raise ValueError(f"{path} is not an hmclab_gb300 sampler checkpoint")
        if int(ck["dimensions"]) != distribution.dimensions:
            raise ValueError(f"checkpoint has {int(ck['dimensions'])} dimensions, the target {distribution.dimensions}")
        C = int(ck["chains"])
        if a["chains"] is not None and int(a["chains"]) != C:
            raise ValueError(f"checkpoint has {C} chains, {a['chains']} were requested")
        if a["dtype"] is not None and _dev.normalise_dtype(a["dtype"]) != str(ck["dtype"]):
            raise ValueError(f"checkpoint chains are {ck['dtype']}, {a['dtype']} was requested")
        if a["initial_model"] is not None:
            raise ValueError("`initial_model` and `resume` exclude each other: the checkpoint holds the positions")
        if a["rng_streams"] is not None:
            raise ValueError("resuming continues the Philox streams; injected `rng_streams` cannot be resumed")
        done = int(ck["proposals_done"])
        thin = int(a["online_thinning"])
        if done % thin:
            raise ValueError(f"the checkpoint's {done} proposals are not a multiple of online_thinning = {thin}")
        a["initial_model"] = ck["q"]
        a["stepsize"] = ck["eps"] if C > 1 else float(ck["eps"][0])
        a["chains"] = C
        a["dtype"] = str(ck["dtype"])
        return ck

    def _recorded(self, n0, n):
        """(first thinned-sample number, count) of the samples recorded by
        this run's proposals [n0, n0 + n): proposal g (counted from the first
        proposal of the chains, a resumed run included) is recorded when
        g % online_thinning == 0, as sample g // online_thinning."""
        t = self.online_thinning
        g0 = self._proposal_base + n0
        first = -(-g0 // t)
        return first, -(-(g0 + n) // t) - first

    def _ring_index(self, first, m):
        """Ring slots of thinned samples first .. first + m - 1 (the device
        indexes the ring by the sample number, modulo its slots)."""
        idx = (first + _numpy.arange(m)) % self.ring_slots
        if m == 0 or (idx[0] == 0 and m <= self.ring_slots and _numpy.all(_numpy.diff(idx) == 1)):
            return slice(0, m)
        return _torch.from_numpy(idx).to(self.device)

    def _parse_surrogate(self, surrogate, training_set, refresh_interval=None, refresh_steps=300, refresh_lr=2e-4):
        self.surrogate = surrogate
        self.training_set = training_set
        self.refresh_interval = None
        if refresh_interval is not None:
            assert surrogate is not None and training_set is not None, (
                "`refresh_interval` needs a surrogate and a training_set to append to")
            assert type(refresh_interval) == int and refresh_interval > 0, "refresh_interval must be a positive int"
            self.refresh_interval = refresh_interval
            self.refresh_steps, self.refresh_lr = int(refresh_steps), float(refresh_lr)
            self.refreshes = 0
        for obj, what in ((surrogate, "surrogate"), (training_set, "training_set")):
            if obj is None:
                continue
            assert self.dtype == "float32", f"`{what}` needs float32 chains"
            assert obj.d == self.dimensions, f"`{what}` has {obj.d} dimensions, the target {self.dimensions}"
        if surrogate is not None:
            assert surrogate.frozen, "freeze() the surrogate before sampling with it (the chain must see a fixed field)"
        if training_set is not None or not self.distribution.graph_safe:
            self.use_graph = False

    def _parse_tempering(self, temperatures, exchange_interval, exchange_streams=None):
        self._temperatures = None
        if temperatures is not None:
            t = _numpy.asarray(temperatures, dtype=_numpy.float64).reshape(-1)
            assert t.size == self.chains, "one temperature per chain is required"
            assert _numpy.all(t > 0) and _numpy.all(_numpy.isfinite(t)), "temperatures must be positive and finite"
            self._temperatures = t
        self.exchange_interval = None
        if exchange_interval is not None:
            assert type(exchange_interval) == int and exchange_interval > 0, "exchange_interval must be a positive int"
            assert self.chains >= 2, "replica exchange needs at least two chains"
            assert exchange_interval % self.online_thinning == 0, (
                "exchange_interval must be a multiple of online_thinning")
            self.exchange_interval = exchange_interval
            # exchanges happen between graph blocks: one block per interval
            self.proposals_per_graph = exchange_interval
        self._exchange_streams = None
        if exchange_streams is not None:
            assert exchange_interval is not None, "`exchange_streams` needs an exchange_interval"
            sched, uu = exchange_streams
            sched = _numpy.asarray(sched, _numpy.int64)
            uu = _numpy.asarray(uu, _numpy.float64)
            npairs = self.chains // 2
            assert sched.ndim == 2 and sched.shape[1] == 2 * npairs, "exchange schedule rows hold 2 * (C // 2) chains"
            assert uu.shape == (sched.shape[0], npairs), "one exchange uniform per pair and schedule row"
            assert all(len(set(r)) == len(r) and r.min() >= 0 and r.max() < self.chains for r in sched), (
                "every schedule row must list distinct chains")
            self._exchange_streams = (sched, uu)

    def _exchange(self, h, n_last):
        """Pair the chains at random and let each pair swap models, after
        proposal n_last (a multiple of exchange_interval).  The pairing is the
        reference's schedule row (Samplers.py:1872-1885): 2 floor(C / 2)
        distinct chains drawn without replacement, consecutive entries
        paired; injected `exchange_streams` replace the draws."""
        C = self.chains
        npairs = C // 2
        if self._exchange_streams is not None:
            sched, uu = self._exchange_streams
            row = n_last // self.exchange_interval
            if row >= len(sched):
                return
            perm = _numpy.asarray(sched[row], _numpy.int32)
            u = _numpy.asarray(uu[row], _numpy.float64)
        else:
            perm = self.rng.choice(C, 2 * npairs, replace=False).astype(_numpy.int32)
            u = self.rng.uniform(0, 1, size=npairs)
        with _torch.cuda.stream(self.stream):
            self._ex_pairs[: 2 * npairs].copy_(_torch.from_numpy(perm))
            self._ex_u[:npairs].copy_(_torch.from_numpy(u))
        _lib.call("hmc_exchange", self._state_ref, npairs, self._ex_pairs.data_ptr(), self._ex_u.data_ptr(),
                  self._ex_swapped.data_ptr(), self._ex_total.data_ptr(), h)

    def run(self, n_proposals):
        """Enqueue the next `n_proposals` proposals (whole graph blocks where
        possible) on the sampler's stream; returns the number issued.  Does not
        synchronise unless samples are drained to files."""
        h = self.stream.cuda_stream
        k = self.proposals_per_graph
        target = min(self.proposals, self._done + int(n_proposals))
        issued = 0
        while self._done < target:
            n = min(k, target - self._done)
            if self.exchange_interval is not None:
                # blocks end right after the proposals that exchange (indices
                # that are multiples of the interval, the first one included)
                g = self._proposal_base + self._done
                nxt = -(-g // self.exchange_interval) * self.exchange_interval
                n = min(n, nxt - g + 1)
            if self.refresh_interval is not None:
                n = min(n, self.refresh_interval - self._done % self.refresh_interval)
            self._load_streams(self._done, n)
            if self._persistent is not None:
                self._persistent.run(n, h)
            elif self.use_graph and n == k:
                if self._graph is None:
                    _lib.call("hmc_graph_begin", h)
                    try:
                        self._issue_block(k, h)
                    finally:
                        exec_ptr = _ct.c_void_p()
                        rc = _lib.load().hmc_graph_end(h, _ct.byref(exec_ptr))
                    _lib.check(rc, "hmc_graph_end")
                    self._graph = exec_ptr
                _lib.call("hmc_graph_launch", self._graph, h)
            else:
                self._issue_block(n, h)
            n_last = self._proposal_base + self._done + n - 1
            if self.exchange_interval is not None and n_last % self.exchange_interval == 0:
                with self._phase("exchange"):
                    self._exchange(h, n_last)
            if self._timers is not None:
                t0 = _time.perf_counter()
                self._drain(self._done, n)
                self._timers["samples.append"].add_host_seconds(_time.perf_counter() - t0)
                for timer in self._timers.values():
                    timer.collect()
            else:
                self._drain(self._done, n)
            self._done += n
            issued += n
            if self.refresh_interval is not None and self._done % self.refresh_interval == 0 and self._done < self.proposals:
                self._refresh(h)
        return issued

    def _refresh(self, h):
        """Exact gradient (and misfit) at every chain's current position into
        the training set, then more training of the surrogate (see
        `refresh_interval`)."""
        dist, dt = self.distribution, self.dtype
        dist._device_gradient(self.q_cur, self.g, False, dt, h)
        tx = None
        if self.training_set.with_values:
            tx = self._training_x
            dist._device_misfit_after_gradient(self.q_cur, tx, False, dt, h)
        if not self.training_set.record(self.q_cur, self.g, h, tx):
            return  # the training set is full: keep the network as it is
        self.surrogate.refresh(self.training_set, steps=self.refresh_steps, lr=self.refresh_lr,
                               seed=self.refreshes, stream=self.stream)
        self.refreshes += 1

    def get_diagnostics(self):
        """The phase timers of diagnostic_mode (reference `Samplers.py:759-764`)."""
        from hmclab_gb300.Helpers.CustomExceptions import InvalidCaseError

        if not self.diagnostic_mode:
            raise InvalidCaseError("Can't return diagnostics if sampler is not in diagnostic mode")
        return list(self._timers.values())

    def _print_diagnostics(self):
        total = self.runtime_seconds
        print("Detailed statistics:")
        print(f"Total runtime: {total:.2f} seconds")
        print()
        print("Device time per phase (CUDA events on the sampler stream):")
        print("{:<30} {:<12} {:<30}".format("Phase", "calls", "percentage of time"))
        for timer in self._timers.values():
            pct = 100.0 * timer.time_spent / total if total > 0 else 0.0
            print("{:<30} {:<12} {:<30.2f}".format(timer.function.__name__, timer.calls, pct))

    def finish(self):
        """Synchronise, release the graph, write attributes and close files."""
        self.stream.synchronize()
        self._end_time = _datetime.now()
        self.runtime_seconds = _time.time() - self._t0
        self.kernel_launches = _lib.launch_count() - self._launches0
        self.proposals_done = self._done
        if self._graph is not None:
            _lib.call("hmc_graph_destroy", self._graph)
            self._graph = None
        if self._fused is not None:
            self._fused.ops.check_status()
        check = getattr(self.distribution, "check_device_status", None)
        if check is not None:
            check()
        self._finalise(self._done)
        if self._timers is not None:
            for timer in self._timers.values():
                timer.collect()
            self._print_diagnostics()
        return self

    def _run(self):
        deadline = self._t0 + self.max_time if self.max_time is not None else None
        try:
            while self._done < self.proposals:
                self.run(self.proposals_per_graph)
                if deadline is not None and _time.time() > deadline:
                    self.stream.synchronize()
                    raise TimeoutError
        except TimeoutError:
            pass
        except KeyboardInterrupt:
            pass
        finally:
            self.finish()

    def _finalise(self, done):
        C = self.chains
        self.exchanges_accepted = int(self._ex_total.cpu()[0]) if self.exchange_interval is not None else 0
        self.current_proposal = max(done - 1, 0)
        acc = self.accepted.cpu().numpy()
        self.accepted_proposals = int(acc[0]) if C == 1 else acc
        q = self.q_cur.to(_torch.float64).cpu().numpy()
        self.current_model = q
        x = self.x_cur.cpu().numpy()
        self.current_x = float(x[0]) if C == 1 else x
        eps = self.eps.to(_torch.float64).cpu().numpy()
        if self.autotuning:
            self.stepsize = float(eps[0]) if C == 1 else eps
            n = self.current_proposal  # the reference keeps [:current_proposal]
            b = self._proposal_base  # records are indexed by the global proposal count
            se = self.rec_eps[b:b + n].cpu().numpy()
            ra = self.rec_acc[b:b + n].cpu().numpy()
            self.stepsizes = se if C > 1 else se[:, :1]
            self.acceptance_rates = ra if C > 1 else ra[:, :1]
        rate = acc / max(done, 1)
        self.acceptance_rate = rate
        if self._writers is not None:
            for c, w in enumerate(self._writers):
                w.write_attribute("acceptance_rate", float(rate[c]))
                w.write_attribute("end_time", self._end_time.strftime("%d-%b-%Y (%H:%M:%S.%f)"))
                w.write_attribute("runtime", str(self._end_time - self._start_time))
                w.write_attribute("runtime_seconds", (self._end_time - self._start_time).total_seconds())
                if self.autotuning:
                    w.write_attribute("acceptance_rates", self.acceptance_rates[:, c : c + 1])
                    w.write_attribute("stepsizes", self.stepsizes[:, c : c + 1])
                w.close()
            self._writers = None
        if self.keep_samples:
            first, m = self._recorded(0, done)
            sel = self._ring_index(first, m)
            self.samples_device = (self.ring_q[sel], self.ring_x[sel])

    # ------------------------------------------------------------------
    def samples_numpy(self, chain=None):
        """Samples kept on the device as (d+1, N) per chain (reference layout);
        (C, d+1, N) for all chains when `chain` is None."""
        assert self.samples_device is not None, "sample(..., keep_samples=True) keeps samples on the device"
        q, x = self.samples_device
        q = q.to(_torch.float64).cpu().numpy()  # N, d, C
        x = x.cpu().numpy()  # N, C
        full = _numpy.concatenate([_numpy.transpose(q, (2, 1, 0)), x.T[:, None, :]], axis=1)
        return full if chain is None else full[chain]

    def samples_host(self):
        """Samples kept on the device, copied to host memory in the device
        layout: q [N][d][C] (state dtype) and misfits x [N][C] (float64)."""
        assert self.samples_device is not None, "sample(..., keep_samples=True) keeps samples on the device"
        q, x = self.samples_device
        hq = _torch.empty(q.shape, dtype=q.dtype, pin_memory=True)
        hx = _torch.empty(x.shape, dtype=x.dtype, pin_memory=True)
        with _torch.cuda.stream(self.stream):
            hq.copy_(q, non_blocking=True)
            hx.copy_(x, non_blocking=True)
        self.stream.synchronize()
        return hq.numpy(), hx.numpy()

    def load_results(self, burn_in: int = 0, chain: int = 0):
        assert burn_in >= 0
        names = self._filenames()
        assert names is not None, "no samples file was written"
        with _Samples(names[chain], burn_in=burn_in) as s:
            return _numpy.array(s.numpy)


def run_together(samplers, n_proposals, warps_per_block=None):
    """Advance several prepared `HMC` samplers (`HMC.prepare`) whose targets
    are small dense linear-Gaussian posteriors of different dimensions by
    `n_proposals` proposals each, all of them in one persistent launch per
    block of proposals; finish each with `finish()` afterwards.  Returns the
    chains per block that were used."""
    from hmclab_gb300._persistent import run_groups

    return run_groups(samplers, n_proposals, warps_per_block)
