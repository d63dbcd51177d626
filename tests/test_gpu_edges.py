"""Edge cases of the CUDA path against the FP64 oracle at fixed iteration
counts: the smallest and largest group counts (1 group: one pair, its
second member padding; 384 = 32 lanes x 6 pairs x 2, the widest sweep
instance and the widest row kernels), a group count whose last pair is
ragged at every lane width, tracks with no segments, a region no track
crosses (volume 0, whose flux add-source keeps finite), and the same through
a server pool.
"""
import numpy as np
import pytest

from openmoc_gb300 import GB300Solver, lattice
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def max_rel(a, b, floor=1e-6):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor * np.abs(b).max())))


def _against_oracle(p, iters=12, shape=None, keff_tol=2e-6, flux_tol=2e-5):
    s = GB300Solver(p)
    if shape:
        s.setSweepShape(*shape)
    s.setConvergenceThreshold(1e-30)
    s.computeEigenvalue(iters)
    o = Oracle(p, "f64", num_threads=8)
    o.compute_eigenvalue(iters, 1, 1e-30)
    assert s.getNumIterations() == iters
    assert abs(s.getKeff() - o.keff) <= keff_tol * o.keff, (s.getKeff(), o.keff)
    assert max_rel(s.getFluxes(), o.phi.reshape(p.num_fsrs, p.num_groups)) <= flux_tol
    s.close()
    return o


@pytest.mark.parametrize("G,shape", [(1, (1, 1)), (1, None), (3, (2, 1)), (33, (4, 5)),
                                     (33, (16, 2)), (384, (32, 6))])
def test_group_counts_at_the_limits(G, shape):
    """1 group (a pair whose second member is padding), 3 and 33 groups (a
    ragged last pair at every lane width), 384 groups (32 lanes x 6 pairs,
    the widest instance; 12 groups per lane in the row kernels)."""
    p = lattice.pin_cell(G, 8, 0.1)
    _against_oracle(p, iters=8 if G == 384 else 12, shape=shape)


def _with_empty_track_and_region(q):
    """q (modified in place) plus a track with no segments (vacuum at both
    ends, linked to itself) and an FSR of the first material that no track
    crosses."""
    T, R = q.num_tracks, q.num_fsrs
    q.seg_off = np.append(q.seg_off, q.seg_off[-1])
    q.track_ang = np.append(q.track_ang, 0).astype(np.int32)
    q.next = np.append(q.next, [T, T]).astype(np.int64)
    q.flags = np.append(q.flags, 0).astype(np.uint8)
    q.fsr_mat = np.append(q.fsr_mat, 0).astype(np.int32)
    q.fsr_vol = np.append(q.fsr_vol, 0.0).astype(np.float32)
    q.num_tracks, q.num_fsrs = T + 1, R + 1
    q.validate()
    return q.contiguous()


def test_tracks_without_segments_and_uncrossed_region():
    p = _with_empty_track_and_region(lattice.pin_cell(7, 8, 0.1))
    o = _against_oracle(p)
    phi = o.phi.reshape(p.num_fsrs, p.num_groups)
    assert np.all(np.isfinite(phi))


def test_edge_problems_through_a_pool():
    """The one-group and the empty-track problems solved in one server pool
    each, alongside a regular problem, give the single solver's result."""
    from openmoc_gb300.serving import Server, pool_capacity
    probs = [lattice.pin_cell(1, 8, 0.1),
             _with_empty_track_and_region(lattice.pin_cell(7, 8, 0.1)),
             lattice.pin_cell(7, 16, 0.1)]
    ref = []
    for p in probs:
        s = GB300Solver(p)
        s.setConvergenceThreshold(1e-30)
        s.useExponentialIntrinsic()
        s.computeEigenvalue(20)
        ref.append((s.getKeff(), s.getFluxes()))
        s.close()
    srv = Server()
    srv.add_pool(1, probs[0].num_polar_half, **pool_capacity(probs[:1], 2))
    srv.add_pool(7, probs[1].num_polar_half, **pool_capacity(probs[1:], 2))
    tickets = [srv.submit(p, max_iters=20, threshold=1e-30) for p in probs]
    srv.run_until_idle()
    for t, (k, f) in zip(tickets, ref):
        r = srv.wait(t, timeout=0)
        assert r["iterations"] == 20
        assert abs(r["keff"] - k) < 1e-6
        assert max_rel(r["flux"], f) < 2e-5
    srv.close()
