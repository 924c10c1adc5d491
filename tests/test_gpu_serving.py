"""Serving pool on the GPU: pooled solves give the same results as the plain public API
with the two-pass kernels (bit for bit: the per-cell arithmetic is the same code), alone
or in a mix, under a budget that admits one at a time or all at once; contexts are
locked while pooled.  Against the default (fused) wakesolve they agree to rounding."""

import numpy as np
import pytest
import torch

import wakis_gb300._native as nat
from wakis_gb300 import serving as S

pytestmark = pytest.mark.gpu

KEYS = ("s", "WP", "WPx", "WPy", "f", "Z", "Zx", "Zy")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def small_requests():
    # Nx = 16, 18, 21: vector widths 4, 2 and 1 in the pooled passes; PEC and lossy walls
    return [S.CavityRequest(tag=0, side=20e-3, rp=4e-3, n=16, sigmaz=6e-3, sigma=0.0, wakelength=0.06),
            S.CavityRequest(tag=1, side=24e-3, rp=5e-3, n=18, sigmaz=7e-3, sigma=2e4, wakelength=0.05),
            S.CavityRequest(tag=2, side=22e-3, rp=3e-3, n=21, sigmaz=5e-3, sigma=0.0, wakelength=0.04),
            S.CavityRequest(tag=3, side=30e-3, rp=6e-3, n=24, sigmaz=8e-3, sigma=5e5, wakelength=0.05)]


@pytest.fixture(scope="module")
def alone():
    return {r.tag: S.solve_alone(r, np.float32, kernels="direct") for r in small_requests()}


def assert_same(got, ref):
    for k in KEYS:
        np.testing.assert_array_equal(np.asarray(got[k]), np.asarray(ref[k]), err_msg=k)


def test_pooled_mix_matches_wakesolve(alone):
    loop = S.ServingLoop(budget_bytes=8 << 30, chunk_steps=16, kernels="direct")
    try:
        recs, summ = loop.run(small_requests())
    finally:
        loop.close()
    assert summ["solves"] == 4
    for tag, ref in alone.items():
        assert_same(loop.results[tag], ref)
    assert {r["tag"]: r["steps"] for r in recs} == {t: alone[t]["Nt"] for t in alone}


def test_pooled_results_match_the_default_wakesolve_to_rounding():
    """The pool's fused kernel (kernels='auto': even Nx) against the default wakesolve
    (the single-grid fused kernel there); odd Nx runs the two-pass kernels on both sides."""
    for req in small_requests():
        ref = S.solve_alone(req, np.float32)
        pool = nat.Pool(1 << 30, chunk_steps=32)
        job = S.ServedSolve(req, kernels="auto")
        try:
            job.submit(pool)
            while not pool.poll(wait_ms=100):
                pass
            got = job.finish()
        finally:
            pool.close()
            job.close()
        for k in ("WP", "Z"):
            a, b = np.asarray(got[k]), np.asarray(ref[k])
            assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b), k


def test_solves_submitted_together_share_chunks(alone):
    """All solves built first, then submitted back to back: they run in the same chunks."""
    jobs = [S.ServedSolve(r, kernels="direct") for r in small_requests()]
    pool = nat.Pool(8 << 30, chunk_steps=8)
    try:
        for j in jobs:
            j.submit(pool)
        done = []
        while len(done) < len(jobs):
            done += pool.poll(wait_ms=200)
        st = pool.stats()
    finally:
        pool.close()
    assert all(d["status"] == 0 for d in done)
    assert st["max_active"] >= 2
    assert st["cell_updates"] == sum(j.req.cells * (j.Nt - j.first) for j in jobs)
    for j in jobs:
        assert_same(j.finish(), alone[j.req.tag])
        j.close()


def test_one_at_a_time_budget_gives_the_same_results(alone):
    reqs = small_requests()
    biggest = max(S.footprint_bytes(r, kernels="direct") for r in reqs)
    loop = S.ServingLoop(budget_bytes=biggest, chunk_steps=64, kernels="direct")
    try:
        recs, summ = loop.run(reqs)
    finally:
        loop.close()
    assert summ["pool"]["max_active"] == 1
    assert summ["pool"]["reserved_bytes"] == 0
    for tag, ref in alone.items():
        assert_same(loop.results[tag], ref)


def test_staggered_arrivals_join_running_solves(alone):
    reqs = small_requests()
    for i, r in enumerate(reqs):
        r.arrival = 0.02 * i
    loop = S.ServingLoop(budget_bytes=8 << 30, chunk_steps=4, kernels="direct")
    try:
        recs, summ = loop.run(reqs)
    finally:
        loop.close()
    for tag, ref in alone.items():
        assert_same(loop.results[tag], ref)
    assert all(r["tti_s"] >= 0 for r in recs)


def test_context_is_locked_while_pooled():
    req = S.CavityRequest(tag=7, side=40e-3, rp=5e-3, n=64, sigmaz=6e-3, sigma=0.0, wakelength=1.0)
    pool = nat.Pool(8 << 30, chunk_steps=64)
    job = S.ServedSolve(req)
    try:
        job.submit(pool)
        with pytest.raises(nat.FitError) as e:
            job.solver._ctx.call("fit_zero_ghosts")
        assert e.value.code == -3
        with pytest.raises(nat.FitError):
            job.submit(pool)
        done = []
        while not done:
            done = pool.poll(wait_ms=200)
        assert done[0]["tag"] == 7 and done[0]["status"] == 0 and done[0]["steps"] == job.Nt - job.first
        job.solver._ctx.call("fit_check_error")  # usable again
        res = job.finish()
        assert np.isfinite(res["WP"]).all()
    finally:
        pool.close()
        job.close()


def test_pool_rejects_fp64_contexts():
    req = S.CavityRequest(tag=0, side=20e-3, rp=4e-3, n=16, sigmaz=6e-3, sigma=0.0, wakelength=0.05)
    pool = nat.Pool(1 << 30)
    job = S.ServedSolve(req, dtype=np.float64)
    try:
        with pytest.raises(nat.FitError) as e:
            job.submit(pool)
        assert e.value.code == -1
        with pytest.raises(nat.FitError):
            pool.reserve(4 << 30)  # larger than the whole budget
        assert pool.reserve(1 << 29)
        assert not pool.reserve(1 << 30)
        pool.release(1 << 29)
    finally:
        pool.close()
        job.close()


def test_fused_pool_mix_with_odd_step_counts():
    """Fused rows (even Nx) next to two-pass rows in one mix, chunk lengths that end
    instances inside a chunk, odd step counts (the first step is taken at submission):
    every result agrees with its default wakesolve to rounding."""
    reqs = small_requests()
    refs = {r.tag: S.solve_alone(r, np.float32) for r in reqs}
    # even Nx: fused rows; the autotuner's choice between fused and two-pass on these
    # small grids depends on timing, so the mix is set explicitly
    jobs = [S.ServedSolve(r, kernels="fused" if r.n % 2 == 0 else "direct") for r in reqs]
    assert [j.solver.kernels for j in jobs] == ["fused", "fused", "direct", "fused"]
    pool = nat.Pool(8 << 30, chunk_steps=6)
    try:
        for j in jobs:
            j.submit(pool)
        done = []
        while len(done) < len(jobs):
            done += pool.poll(wait_ms=100)
    finally:
        pool.close()
    assert all(d["status"] == 0 for d in done)
    assert {d["tag"]: d["steps"] for d in done} == {j.req.tag: j.Nt - j.first for j in jobs}
    for j in jobs:
        got = j.finish()
        for k in ("WP", "Z", "WPx"):
            a, b = np.asarray(got[k]), np.asarray(refs[j.req.tag][k])
            assert np.linalg.norm(a - b) <= 1e-5 * max(np.linalg.norm(b), 1e-30), (j.req.tag, k)
        j.close()


def _run_pool(jobs, chunk_steps, variants=None):
    pool = nat.Pool(8 << 30, chunk_steps=chunk_steps)
    try:
        for vec, minb in (variants or {}).items():
            pool.tune_fused(vec, minb)
        for j in jobs:
            j.submit(pool)
        done = []
        while len(done) < len(jobs):
            done += pool.poll(wait_ms=100)
        stats = pool.stats()
    finally:
        pool.close()
    assert all(d["status"] == 0 for d in done), done
    return stats


def test_fused_pool_equals_two_pass_wakesolve_bitwise(alone):
    """The pool's fused step on plane segments, every vector width (Nx = 16 and 24:
    4-wide, 18: 2-wide, 21: single cells), gives the two-pass wakesolve's results bit for
    bit: the per-cell arithmetic is the same code, and the cells before a segment (the
    previous plane's last row here, one segment per plane) are recomputed exactly."""
    reqs = small_requests()
    jobs = [S.ServedSolve(r, kernels="fused") for r in reqs]
    stats = _run_pool(jobs, chunk_steps=8)
    assert stats["fused_cell_updates"] == stats["cell_updates"] > 0
    for j in jobs:
        assert_same(j.finish(), alone[j.req.tag])
        j.close()


@pytest.mark.parametrize("choice", [0, 1])
def test_fused_pool_multi_segment_planes_bitwise(choice):
    """Planes of several segments (Nx*Ny = 2304 .. 2500 cells, segments of 1024 - Nx
    cells, so the cells before a segment are the previous segment's, in the same plane),
    both compiled register budgets, a chunk length that ends solves inside a chunk: bit for
    bit the two-pass wakesolve."""
    reqs = [S.CavityRequest(tag=10, side=30e-3, rp=5e-3, n=48, sigmaz=8e-3, sigma=0.0, wakelength=0.02),
            S.CavityRequest(tag=11, side=32e-3, rp=6e-3, n=50, sigmaz=9e-3, sigma=3e4, wakelength=0.02),
            S.CavityRequest(tag=12, side=28e-3, rp=4e-3, n=49, sigmaz=7e-3, sigma=0.0, wakelength=0.02)]
    refs = {r.tag: S.solve_alone(r, np.float32, kernels="direct") for r in reqs}
    jobs = [S.ServedSolve(r, kernels="fused") for r in reqs]
    variants = {vec: S.POOL_FUSED_VARIANTS[vec][choice] for vec in (4, 2, 1)}
    stats = _run_pool(jobs, chunk_steps=10, variants=variants)
    assert stats["fused_variant"] == variants
    assert stats["fused_cell_updates"] == stats["cell_updates"]
    for j in jobs:
        assert_same(j.finish(), refs[j.req.tag])
        j.close()


def test_fused_pool_rejects_unknown_variant():
    pool = nat.Pool(1 << 30, chunk_steps=8)
    try:
        with pytest.raises(nat.FitError):
            pool.tune_fused(4, 5)
    finally:
        pool.close()
