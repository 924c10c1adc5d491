"""FP64 parity at the full sizes of the benchmark configurations that are too large for
a complete CPU-oracle run inside a test, and the FP32 accuracy of the large pillbox:

* the lossy cavity (128x128x256, sigma = 1e4 walls, 10-cell z PML), both beam runs (beta 1 on
  axis; beta 0.8 with source and test 2 mm off axis): the first 300 steps of the wake
  run in FP64 -- fields E, H and the partial 3x3 wake integral -- against the CPU oracle
  within 1e-10 relative L2, with s, dt and Nt identical;
* the sphere and wave packet (256^3 unit box, 12-cell PML on all faces, eps_r = 2 sphere):
  100 FP64 steps, E_z at the 64 seeded probes after every step and the final fields,
  against the oracle within 1e-10;
* the 512x512x1024 lossy pillbox: the FP32 wake potential over the first 0.3 m
  against the FP64 run at the same time step, within 1e-4 relative L2.

The oracle runs in spawned worker processes started before the first GPU run here, so
the CPU and GPU halves of each comparison overlap.
"""

import concurrent.futures as cf
import multiprocessing as mp
import os
import sys

import numpy as np
import pytest
import torch

import cases as C
from oracle_runner import rel_l2, run_oracle_probes, run_oracle_wake_partial
from product_runner import run_case, run_wake_partial

pytestmark = pytest.mark.gpu

WAKE_STEPS = 300   # lossy cavity: steps of the partial wake run
PROBE_STEPS = 100  # sphere and wave packet: steps of the probe run
TOL64 = 1e-10      # FP64 GPU against the FP64 oracle (relative L2)
TOL_WP32 = 1e-4    # FP32 wake potential against FP64 (relative L2)


def _fp64(name):
    return dict(C.WORKLOADS[name], dtype="float64")


@pytest.fixture(scope="module")
def oracle_jobs():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    ex = cf.ProcessPoolExecutor(max_workers=3, mp_context=mp.get_context("spawn"))
    jobs = {name: ex.submit(run_oracle_wake_partial, _fp64(name), WAKE_STEPS) for name in ("lossy_cavity_128x128x256", "lossy_cavity_128x128x256_offset")}
    jobs["sphere_packet_256"] = ex.submit(run_oracle_probes, _fp64("sphere_packet_256"), PROBE_STEPS)
    yield jobs
    ex.shutdown(wait=True, cancel_futures=True)


@pytest.mark.parametrize("name", ["lossy_cavity_128x128x256", "lossy_cavity_128x128x256_offset"])
def test_lossy_cavity_fp64_partial_wake_matches_oracle(name, oracle_jobs, tmp_path):
    got = run_wake_partial(_fp64(name), WAKE_STEPS, tmpdir=tmp_path, dtype=np.float64)
    torch.cuda.synchronize()
    ref = oracle_jobs[name].result()
    assert int(got["Nt"]) == int(ref["Nt"])
    assert got["dt"] == ref["dt"]
    np.testing.assert_array_equal(got["s"], ref["s"])
    assert np.count_nonzero(ref["WP_3d"][4]) > 0  # the partial integral is not empty
    for k in ("E", "H"):
        assert rel_l2(got[k], ref[k]) < TOL64, (k, rel_l2(got[k], ref[k]))
    for li in range(9):
        e = rel_l2(got["WP_3d"][li], ref["WP_3d"][li])
        assert e < TOL64, (li, e)


def test_sphere_packet_fp64_probes_match_oracle(oracle_jobs, tmp_path):
    case = dict(_fp64("sphere_packet_256"), Nt=PROBE_STEPS)
    got = run_case("sphere_packet_256", case=case, tmpdir=tmp_path, dtype=np.float64)
    torch.cuda.synchronize()
    ref = oracle_jobs["sphere_packet_256"].result()
    assert got["dt"] == ref["dt"]
    assert got["probes"].shape == ref["probes"].shape == (PROBE_STEPS, 64)
    assert np.abs(ref["probes"]).max() > 0
    for k in ("probes", "E", "H"):
        assert rel_l2(got[k], ref[k]) < TOL64, (k, rel_l2(got[k], ref[k]))


def test_pillbox_fp32_wake_against_fp64():
    """The 268M-cell pillbox: FP32 fields (FP64 coefficients, compensated FP64 wake sums
    and DFT) against the FP64 path at the FP32 run's time step, WP over 0.3 m."""
    import gc

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import wakis_gb300 as wg
    from bench import Pillbox

    P = Pillbox()
    res = {}
    dt = None
    for key, dtype in (("fp32", np.float32), ("fp64", np.float64)):
        mask = P.walls_mask(device=torch.device("cuda", 0))
        grid, wake, s = P.build(wg, mask, dtype=dtype, dt=dt)
        dt = float(s.dt)
        del mask
        s.wakesolve(wakelength=P.wakelength)
        res[key] = dict(s=wake.s, WP=wake.WP, Nt=s.Nt)
        del s, grid, wake
        gc.collect()
        torch.cuda.empty_cache()
    a, b = res["fp32"], res["fp64"]
    assert a["Nt"] == b["Nt"]
    np.testing.assert_array_equal(a["s"], b["s"])
    e = rel_l2(a["WP"], b["WP"])
    assert e < TOL_WP32, e
