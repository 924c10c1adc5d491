"""Failure paths, exercised without faulting, trapping or hanging the GPU.

Device side: the kernels that wait on bulk or tensor copies (the staged passes and the
TMA-fed fused step) take a run-time limit on their polls.  With the limit set to 0 every
wait gives up at once: the kernel records FIT_ERR_TIMEOUT in the context's error word,
still waits (bounded) for the copies it issued, and returns.  The host reads the word
(fit_check_error, called at the end of every device loop) and raises; a following normal
run on the same context matches the oracle.

Host side (the serving loop): a request whose footprint exceeds the whole budget is
rejected on arrival, a request cancelled while queued or while its chunks run is handed
back by the pool, and a request whose read-back results are not finite fails; each ends
with its own status while every other request of the mix completes with the results of
solving it alone, bit for bit.  The per-request JSONL trace records every request.
"""

import json

import numpy as np
import pytest
import torch

import cases as C
import wakis_gb300._native as nat
from oracle_runner import rel_l2, run_oracle_case
from product_runner import run_case
from wakis_gb300 import serving as S

pytestmark = pytest.mark.gpu

KEYS = ("s", "WP", "WPx", "WPy", "f", "Z", "Zx", "Zy")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def _random_solver(kernels, dtype=np.float32):
    import wakis_gb300 as wg
    g = wg.GridFIT3D(-1, 1, -1, 1, -1, 1, 16, 12, 24, verbose=0)
    s = wg.SolverFIT3D(g, cfln=0.5, bc_low=["pec"] * 3, bc_high=["pec"] * 3, bg=[1.0, 1.0, 0.2], dtype=dtype,
                       verbose=0)
    s.kernels = kernels
    rng = np.random.default_rng(1)
    s.E.fromarray(rng.standard_normal(3 * s.N).astype(dtype))
    s.H.fromarray(rng.standard_normal(3 * s.N).astype(dtype))
    return s


def _ghost_free(s, rng):
    """Random E, H with the ghost components of the last index planes zero (what the first
    step of a fresh solver leaves), so a solver that already took its first step and a
    fresh one start from the same state."""
    E = rng.standard_normal((3, s.Nz, s.Ny, s.Nx)).astype(np.float32)
    H = rng.standard_normal((3, s.Nz, s.Ny, s.Nx)).astype(np.float32)
    E[0, :, :, -1] = 0
    E[1, :, -1, :] = 0
    E[2, -1, :, :] = 0
    H[0, :, -1, :] = 0
    H[0, -1, :, :] = 0
    H[1, :, :, -1] = 0
    H[1, -1, :, :] = 0
    H[2, :, :, -1] = 0
    H[2, :, -1, :] = 0
    return E.ravel(), H.ravel()


@pytest.mark.parametrize("kernels,staging", [("staged", "0"), ("fused", "1")])
def test_wait_limit_zero_reports_timeout_and_context_recovers(kernels, staging):
    s = _random_solver(kernels)
    s.fused_staging = staging
    s._ctx.call("fit_set_wait_limit", 0)
    with pytest.raises(nat.FitError) as ei:
        s.emsolve(20)  # first step from the host, then the device loop; both wait on copies
    assert ei.value.code == nat.FIT_ERR_TIMEOUT
    s._ctx.call("fit_check_error")  # reported once: the word is clear again
    # the same context with the default limit: a fresh start matches the two-pass kernels
    s._ctx.call("fit_set_wait_limit", 1 << 24)
    s.reset_fields()
    ref = _random_solver("direct")
    rng = np.random.default_rng(2)
    E0, H0 = _ghost_free(s, rng)
    for x in (s, ref):
        x.E.fromarray(E0)
        x.H.fromarray(H0)
        x.emsolve(20)
    for k in ("E", "H", "J"):
        np.testing.assert_array_equal(getattr(s, k).numpy(), getattr(ref, k).numpy(), err_msg=k)


def test_wait_limit_then_reference_case_matches_oracle(tmp_path, monkeypatch):
    """After a run that gave up, a normal wake run on the TMA-fed step passes the FP64
    oracle at 1e-10."""
    s = _random_solver("fused", np.float64)
    s.fused_staging = "1"
    s._ctx.call("fit_set_wait_limit", 0)
    with pytest.raises(nat.FitError):
        s.emsolve(8)
    monkeypatch.setenv("WAKIS_GB300_KERNELS", "fused")
    monkeypatch.setenv("WAKIS_GB300_STAGING", "1")
    got = run_case("cavity_f64", tmpdir=tmp_path)
    ref = run_oracle_case("cavity_f64")
    for k in ("WP", "Z", "E", "H"):
        assert rel_l2(got[k], ref[k]) < 1e-10, k


def test_wait_limit_rejects_negative():
    s = _random_solver("direct")
    with pytest.raises(nat.FitError):
        s._ctx.call("fit_set_wait_limit", -1)


# ---------------------------------------------------------------- serving loop

def _mix():
    # tags 0..3 complete; 4: footprint above the budget; 5: cancelled while running;
    # 6: cancelled while queued; 7: NaN injected into its read-back results
    base = dict(sigmaz=6e-3, wakelength=0.05)
    reqs = [S.CavityRequest(tag=0, side=20e-3, rp=4e-3, n=16, sigma=0.0, **base),
            S.CavityRequest(tag=1, side=24e-3, rp=5e-3, n=18, sigma=2e4, **base),
            S.CavityRequest(tag=2, side=22e-3, rp=3e-3, n=21, sigma=0.0, **base),
            S.CavityRequest(tag=3, side=30e-3, rp=6e-3, n=24, sigma=5e5, **base),
            S.CavityRequest(tag=4, side=30e-3, rp=6e-3, n=400, sigma=0.0, **base),
            S.CavityRequest(tag=5, side=26e-3, rp=5e-3, n=20, sigma=0.0, sigmaz=6e-3, wakelength=30.0),
            S.CavityRequest(tag=6, side=26e-3, rp=5e-3, n=20, sigma=0.0, arrival=0.0, **base),
            S.CavityRequest(tag=7, side=21e-3, rp=4e-3, n=17, sigma=1e5, **base)]
    return reqs


def test_serving_failures_stay_with_their_request(tmp_path):
    reqs = _mix()
    alone = {r.tag: S.solve_alone(r, np.float32, kernels="direct") for r in reqs if r.tag in (0, 1, 2, 3)}
    trace = tmp_path / "trace.jsonl"
    # the budget holds the small requests, not tag 4 (n = 400)
    loop = S.ServingLoop(budget_bytes=2 << 30, chunk_steps=16, kernels="direct", trace_path=str(trace))
    state = {"cancelled": False}

    def on_tick(lp, now, running):
        if not state["cancelled"]:
            lp.cancel(6)  # still queued or just admitted
            state["cancelled"] = True
        if 5 in running:
            lp.cancel(5)

    def readback(tag, res):
        if tag == 7:
            res["WP"] = np.array(res["WP"], copy=True)
            res["WP"][3] = np.nan

    try:
        recs, summ = loop.run(reqs, on_tick=on_tick, readback_hook=readback)
    finally:
        loop.close()
    status = {r["tag"]: r["status"] for r in recs}
    assert status[4] == "rejected"
    assert status[5] == "cancelled"
    assert status[6] == "cancelled"
    assert status[7] == "failed" and "non-finite" in [r for r in recs if r["tag"] == 7][0]["reason"]
    for tag in (0, 1, 2, 3):
        assert status[tag] == "done"
        for k in KEYS:
            np.testing.assert_array_equal(np.asarray(loop.results[tag][k]), np.asarray(alone[tag][k]), err_msg=k)
    assert summ["solves"] == 4 and summ["failed"] == {"rejected": 1, "failed": 1, "cancelled": 2}
    lines = [json.loads(x) for x in trace.read_text().splitlines()]
    assert sorted(x["tag"] for x in lines) == list(range(8))
    for x in lines:
        if x["status"] == "done":
            assert x["arrival_s"] <= x["admitted_s"] <= x["submitted_s"] <= x["done_s"]
            assert x["pool_submit_ms"] <= x["pool_start_ms"] <= x["pool_done_ms"]


def test_pool_cancel_of_unknown_tag_is_an_argument_error():
    pool = nat.Pool(1 << 28, chunk_steps=8)
    try:
        with pytest.raises(nat.FitError) as ei:
            pool.cancel(12345)
        assert ei.value.code == -1
    finally:
        pool.close()
