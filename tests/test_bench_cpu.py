"""Host logic of bench.py (no GPU): peaks with and without the measured
file, the clock record's parsing, the surrogate trajectory choice and the
FWI workload's algorithmic bytes."""
import json
import os

import pytest

import bench


def test_peaks_measured_and_fallback(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.peaks() == (6800.0, 1900.0, 1700.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6791.0, "bf16_tflops": 1935.3}))
    assert bench.peaks() == (6791.0, 1935.3, 1935.3, "measured")


class _FakeProc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_sampler_parses_nvidia_smi_lines():
    c = bench.ClockSampler(0)
    c.proc = _FakeProc()
    c.lines = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1000.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    r = c.stop()
    assert r == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    assert bench.ClockSampler(0).stop()["reasons"] == ["nvidia-smi unavailable"]


def test_choose_trajectory():
    pilot = [(0.8 * 0.24**2, 2, 0.12, 0.8), (0.3 * 0.48**2, 8, 0.06, 0.3), (0.1 * 0.96**2, 8, 0.12, 0.1)]
    # the last entry has the largest gain but an untrustworthy acceptance
    assert bench.choose_trajectory(pilot) == (8, 0.06)
    assert bench.choose_trajectory(pilot, min_acceptance=0.5) == (2, 0.12)
    assert bench.choose_trajectory([(0.0, 4, 0.03, 0.0), (0.01, 2, 0.06, 0.1)]) == (2, 0.06)


def test_fwi_workload_algorithmic_bytes():
    wl = bench.FwiWorkload()
    assert (wl.cfg.nxc, wl.cfg.nzc) == (240, 140)
    # 20 FP32 words per cell and chain per forward step (velocity + stress)
    assert wl.stencil_bytes_per_step() == 80.0 * 240 * 140 * 64
    cfg = wl.config()
    assert cfg["chains"] == 64 and cfg["nt"] == 1500 and cfg["params"] == 600


def _fake_reference(wl, path, **over):
    import numpy as np

    d = 600
    ref = dict(mean=np.zeros(d), std=np.ones(d), ess=np.full(d, 2000.0), ess_per_chain_proposal=0.15,
               q_final=np.zeros((d, wl.chains)), chains=wl.chains, leapfrog_steps=wl.L, stepsize=wl.stepsize,
               noise_fraction=wl.noise_fraction, seed=0, proposals=200)
    ref.update(over)
    np.savez(path, **ref)
    return str(path)


def test_fwi_reference_fixture_is_checked_against_the_workload(tmp_path):
    wl = bench.FwiWorkload()
    ref, why = bench.load_fwi_reference(wl, str(tmp_path / "missing.npz"))
    assert ref is None and "no reference fixture" in why
    ref, why = bench.load_fwi_reference(wl, _fake_reference(wl, tmp_path / "ok.npz"))
    assert why is None and float(ref["ess_per_chain_proposal"]) == 0.15
    ref, why = bench.load_fwi_reference(wl, _fake_reference(wl, tmp_path / "bad.npz", stepsize=0.2))
    assert ref is None and "stepsize" in why


def test_fwi_headline_validity_gates():
    import numpy as np

    rng = np.random.default_rng(0)
    d = 600
    ref = dict(mean=np.zeros(d), std=np.ones(d), ess=np.full(d, 4000.0))
    ess = np.full(d, 400.0)
    # unbiased run: z ~ N(0, 1)
    mean = rng.normal(size=d) * np.sqrt(1 / 400 + 1 / 4000)
    std = 1 + rng.normal(size=d) * np.sqrt(1 / 800 + 1 / 8000)
    mc = bench.moment_check(mean, std, ess, ref)
    assert mc["mean_z_max"] < 4.5 and mc["std_z_max"] < 4.5
    assert bench.fwi_validity(ess, mc) == []
    # windows that did not truncate are flagged negative by the estimator
    raw = ess.copy()
    raw[:100] *= -1
    assert any("lag windows" in r for r in bench.fwi_validity(raw, mc))
    # a biased run: one parameter's mean off by 10 Monte Carlo errors
    mean_b = mean.copy()
    mean_b[7] += 10 * np.sqrt(1 / 400 + 1 / 4000)
    mc_b = bench.moment_check(mean_b, std, ess, ref)
    assert any("moments disagree" in r for r in bench.fwi_validity(ess, mc_b))
    assert bench.fwi_validity(ess, None) == ["no reference moments to check the run against"]
    assert not mc["within_2pct_of_reference_std"]


def test_variogram_decorrelation_reads_subdiffusive_chains_low():
    """variogram_min = 1 - autocorrelation at the lag, from the mean squared
    displacement over twice the reference variance: an AR(1) chain with
    rho = 0.9 gives 1 - 0.9^lag; a chain whose successive moves undo each
    other (x_t = a_t - a_(t-1) added to a slow AR(1)) moves a lot per step
    but little over many steps."""
    import numpy as np
    import torch

    rng = np.random.default_rng(0)
    N, d, C, rho = 4000, 3, 64, 0.9
    x = np.zeros((N, d, C))
    x[0] = rng.normal(size=(d, C))
    for t in range(1, N):
        x[t] = rho * x[t - 1] + np.sqrt(1 - rho**2) * rng.normal(size=(d, C))
    q = torch.from_numpy(x)
    for lag in (1, 5, 20):
        assert abs(bench.variogram_min(q, np.ones(d), lag) - (1 - rho**lag)) < 0.03
    slow = np.zeros((N, d, C))
    rs = 0.999
    for t in range(1, N):
        slow[t] = rs * slow[t - 1] + np.sqrt(1 - rs**2) * rng.normal(size=(d, C))
    a = 0.1 * rng.normal(size=(N, d, C))
    jitter = a - np.roll(a, 1, axis=0)
    z = torch.from_numpy(slow + jitter)
    one, many = bench.variogram_min(z, np.ones(d), 1), bench.variogram_min(z, np.ones(d), 30)
    # 30 independent moves of the single-step size would reach 30 x `one`
    assert many < 0.5 * 30 * one
