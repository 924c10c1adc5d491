"""GridFIT3D.refine_axis and use_mesh_refinement (wakis/gridFIT3D.py:204-217, 771-920),
pinned to the reference's own refine_axis output on seeded snap sets
(tests/golden/refine_axis.npz, written by tests/golden/make_golden.py).  CPU only: the
refinement is grid set-up (scipy least_squares), before any device work."""

import numpy as np
import pytest

import cases as C
from oracle_runner import load_golden


def _grid():
    import wakis_gb300 as wg
    return wg.GridFIT3D(0, 1, 0, 1, 0, 1, 2, 2, 2, verbose=0)


@pytest.mark.parametrize("i", range(len(C.REFINE_CASES)))
def test_refine_axis_matches_reference(i):
    ref = load_golden("refine_axis")
    seed, lo, hi, n, ns, method = C.REFINE_CASES[i]
    snaps = C.refine_snaps(seed, lo, hi, ns)
    x = _grid().refine_axis(lo, hi, n, snaps, method=method)
    np.testing.assert_array_equal(x, ref[f"x{i}"])
    # the snaps are pulled by a penalty, not held: the reference's nodes land near them
    assert np.all(np.min(np.abs(x[:, None] - snaps[None, :]), axis=0) < 0.5 * (hi - lo) / (n - 1))


def test_refine_axis_subdivision_raises_like_reference():
    ref = load_golden("refine_axis")
    with pytest.raises(Exception) as ei:
        _grid().refine_axis(0.0, 1.0, 11, np.array([0.0, 0.37, 1.0]), method="subdivision")
    assert [type(ei.value).__name__, str(ei.value)] == list(ref["subdivision_exc"])
    with pytest.raises(ValueError):
        _grid().refine_axis(0.0, 1.0, 11, np.array([0.0, 0.37, 1.0]), method="spline")


def test_mesh_refinement_from_snap_points():
    """use_mesh_refinement with snap points: every axis is refine_axis of the snap
    coordinates rounded to 5 decimals plus the domain bounds, as the reference derives them
    from STL edge points."""
    import wakis_gb300 as wg
    pts = np.array([[-0.012, 0.0, -0.031], [0.0, 0.0155, 0.0], [0.0204, 0.0, 0.02713]])
    g = wg.GridFIT3D(-0.03, 0.03, -0.03, 0.03, -0.06, 0.06, 20, 20, 40, use_mesh_refinement=True, snap_points=pts,
                     verbose=0)
    for a, name in enumerate("xyz"):
        lo, hi = getattr(g, name + "min"), getattr(g, name + "max")
        snaps = np.unique(np.concatenate(([lo], np.unique(np.round(pts[:, a], 5)), [hi])))
        n = {"x": 21, "y": 21, "z": 41}[name]
        np.testing.assert_array_equal(getattr(g, name), _grid().refine_axis(lo, hi, n, snaps, tol=1e-8))
        np.testing.assert_array_equal(getattr(g, "d" + name), np.diff(getattr(g, name)))
    assert g.Nx == len(g.x) - 1 and g.Nz == len(g.z) - 1


def test_mesh_refinement_without_snaps_raises_like_reference():
    import wakis_gb300 as wg
    with pytest.raises(AttributeError):
        wg.GridFIT3D(-1, 1, -1, 1, -1, 1, 8, 8, 8, use_mesh_refinement=True, verbose=0)
    with pytest.raises(NotImplementedError):
        wg.GridFIT3D(-1, 1, -1, 1, -1, 1, 8, 8, 8, use_mesh_refinement=True, stl_solids={"a": "a.stl"},
                     verbose=0)


@pytest.mark.gpu
def test_refined_grid_wake_matches_oracle(tmp_path):
    """A wake run of the cavity case on axes refined onto the cube and pipe edges (the
    snap points an STL of that cavity would give) matches the FP64 oracle on the same axes
    at the parity tolerance."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import wakis_gb300 as wg
    from oracle_runner import rel_l2, run_oracle_case
    from product_runner import run_case
    mm = 1e-3
    pts = np.array([[-25 * mm, 0.0, -25 * mm], [25 * mm, 0.0, 25 * mm], [-5 * mm, 0.0, 0.0], [5 * mm, 0.0, 0.0],
                    [0.0, -25 * mm, 0.0], [0.0, 25 * mm, 0.0], [0.0, -5 * mm, 0.0], [0.0, 5 * mm, 0.0]])
    g = wg.GridFIT3D(-30 * mm, 30 * mm, -30 * mm, 30 * mm, -60 * mm, 60 * mm, 16, 16, 32, use_mesh_refinement=True,
                     snap_points=pts, verbose=0)
    assert np.ptp(np.diff(g.z)) > 0  # non-uniform
    case = dict(C.CASES["cavity_f64"], grid=dict(x=g.x, y=g.y, z=g.z))
    got = run_case("refined", case=case, tmpdir=tmp_path)
    ref = run_oracle_case("refined", case=case)
    assert int(got["Nt"]) == int(ref["Nt"])
    np.testing.assert_array_equal(got["s"], ref["s"])
    for k in ("WP", "Z", "E", "H", "WP_3d"):
        assert rel_l2(got[k], ref[k]) < 1e-10, (k, rel_l2(got[k], ref[k]))
