"""Linear-source requests in the batched solve server (CPULSSolver solves in
linear-source pools) on the GPU.

  * OpenMOC's CPULSSolver fixtures (eigenvalue, computeSource, computeFlux
    with fixed source moments and negative fluxes allowed) solved through
    pools: iterations, keff within 1e-5, scalar fluxes within 1e-4 and flux
    moments, as the single-problem linear-source tests ask;
  * a generated lattice through a pool against the FP64 linear-source oracle
    at a fixed iteration count;
  * the same request alone, in a mix of linear-source requests and beside a
    flat-source pool of the same group count, against the single-problem
    GB300LSSolver with the same sweep shape (only the order of the tally
    atomics differs);
  * requests the server must refuse.
"""
import numpy as np
import pytest

from conftest import LS_CASES, load_case
from openmoc_gb300 import lattice
from openmoc_gb300._native import MOCError
from openmoc_gb300.serving import Server, pool_capacity
from openmoc_gb300.solver import EXP_INTRINSIC
from oracle.oracle import LSOracle

pytestmark = pytest.mark.gpu

NEVER = 1e-12   # threshold no solve reaches: stop at the iteration count


def _xyz(xy, R, G):
    """[R][2][G] moments -> [R][3][G] (z = 0)."""
    m = np.zeros((R, 3, G), np.float32)
    m[:, :2, :] = np.asarray(xy, np.float32).reshape(R, 2, G)
    return m


def _rel(got, ref, floor):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    return float(np.max(np.abs(got - ref) /
                        np.maximum(np.abs(ref), floor * np.abs(ref).max())))


def _peak(got, ref):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    return float(np.max(np.abs(got - ref)) / np.abs(ref).max())


def _ls_server(problems, max_solves, shape=None, flat_too=False):
    srv = Server(iterations_per_poll=8)
    by_key = {}
    for p in problems:
        by_key.setdefault((p.num_groups, p.num_polar_half), []).append(p)
    for (G, ph), ps in sorted(by_key.items()):
        cap = pool_capacity(ps, max_solves)
        srv.add_pool(G, ph, shape=shape, linear_source=True, **cap)
        if flat_too:
            srv.add_pool(G, ph, shape=shape, **cap)
    return srv


def _submit_case(srv, p, sc, arr):
    kind = {0: "eigenvalue", 1: "source", 2: "flux"}[int(sc["run_kind"])]
    fsm = None
    if "fixed_source_xy" in arr:
        fsm = _xyz(arr["fixed_source_xy"], p.num_fsrs, p.num_groups)
    return srv.submit(p, kind, int(sc["max_iters"]), int(sc["res_type"]),
                      k_eff=float(sc["k_source"]), threshold=sc["tolerance"],
                      linear_source=True, fixed_source_moments=fsm,
                      allow_negative_fluxes=bool(sc.get("allow_negative", 0)))


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_ls_fixtures_batched_match_openmoc(precision):
    cases = {c: load_case(c, precision) for c in LS_CASES}
    # every case twice: two solves of one problem share the pool
    srv = _ls_server([v[0] for v in cases.values()], 4)
    tickets = {c: [_submit_case(srv, *cases[c]) for _ in range(2)] for c in cases}
    srv.run_until_idle()
    for c, (p, sc, arr) in cases.items():
        R, G = p.num_fsrs, p.num_groups
        for t in tickets[c]:
            r = srv.wait(t, timeout=0)
            assert abs(r["iterations"] - int(sc["iterations"])) <= 1, c
            if int(sc["run_kind"]) == 0:
                assert abs(r["keff"] - sc["keff"]) < 1e-5, (c, r["keff"], sc["keff"])
            assert _rel(r["flux"], arr["flux"].reshape(R, G), 1e-4) < 1e-4, c
            assert _peak(r["moments"], arr["ls_moments"].reshape(R, 3, G)) < 5e-4, c
    st = srv.stats()
    assert st["completed"] == 2 * len(cases) and st["failed"] == 0
    srv.close()


def _lattice_ls(n, G, perturb=None):
    """A vacuum-bounded (+x, +y) n x n lattice with a water centre pin;
    perturb = seed: cross sections perturbed by 5 %."""
    from openmoc_gb300.lattice import REFLECTIVE, VACUUM
    mats = lattice._fuel_mod(7, G, 1, None if perturb is None else (perturb, 0.05))
    pm = np.zeros((n, n), np.int32)
    pm[n // 2, n // 2] = 1
    return lattice.lattice(n, n, pm, mats, 1, num_azim=16, spacing=0.1,
                           linear_source=True,
                           bc=(REFLECTIVE, VACUUM, REFLECTIVE, VACUUM))


def test_ls_pool_matches_oracle():
    """A generated 3 x 3 linear-source lattice solved in a pool (beside
    another request) against the FP64 oracle after 12 eigenvalue
    iterations."""
    G, iters = 7, 12
    p = _lattice_ls(3, G)
    other = _lattice_ls(3, G, perturb=5)
    o = LSOracle(p, p.linear_source, "f64", num_threads=8)
    o.compute_eigenvalue(iters, 1, 1e-30)
    srv = _ls_server([p, other], 2)
    t = srv.submit(p, max_iters=iters, threshold=NEVER, linear_source=True)
    srv.submit(other, max_iters=iters + 5, threshold=NEVER, linear_source=True)
    srv.run_until_idle()
    r = srv.wait(t, timeout=0)
    R = p.num_fsrs
    assert r["iterations"] == iters
    assert abs(r["keff"] - o.keff) < 2e-6
    assert _rel(r["flux"], o.phi.reshape(R, G), 1e-4) < 2e-5
    assert _peak(r["moments"], o.mom.reshape(R, 3, G)) < 1e-4
    srv.close()


@pytest.mark.parametrize("G,shape", [(7, (4, 1)), (16, (8, 1))])
def test_ls_same_result_alone_in_mix_and_single(G, shape):
    from openmoc_gb300 import GB300LSSolver
    iters = 30
    target = _lattice_ls(3, G)
    others = [_lattice_ls(3, G, perturb=11 + i) for i in range(3)]
    s = GB300LSSolver(target, device=0)
    s.setSweepShape(*shape)
    s.setConvergenceThreshold(NEVER)
    s.computeEigenvalue(iters, 1)
    ref = dict(keff=s.getKeff(), flux=s.getFluxes(), moments=s.getFluxMoments())
    s.close()

    def run(with_others, flat_too):
        srv = _ls_server([target] + others, 4, shape=(*shape, EXP_INTRINSIC),
                         flat_too=flat_too)
        ts = []
        if with_others:
            ts += [srv.submit(q, max_iters=iters + 7 * i, threshold=NEVER,
                              linear_source=True) for i, q in enumerate(others)]
            srv.step()                   # the others already running ...
        if flat_too:                     # ... and a flat solve of the same G
            ts.append(srv.submit(others[0], max_iters=iters, threshold=NEVER))
        t = srv.submit(target, max_iters=iters, threshold=NEVER, linear_source=True)
        srv.run_until_idle()
        r = srv.wait(t, timeout=0)
        for u in ts:
            srv.wait(u, timeout=0)
        assert srv.stats()["failed"] == 0
        srv.close()
        return r

    for with_others, flat_too in ((False, False), (True, False), (True, True)):
        r = run(with_others, flat_too)
        assert r["iterations"] == iters
        assert abs(r["keff"] - ref["keff"]) < 1e-6, (with_others, flat_too)
        assert _rel(r["flux"], ref["flux"], 1e-4) < 2e-5, (with_others, flat_too)
        assert _peak(r["moments"], ref["moments"]) < 1e-4, (with_others, flat_too)


def test_ls_requests_refused():
    p = lattice.pin_cell(7, linear_source=True)
    flat_only = Server()
    flat_only.add_pool(7, p.num_polar_half, **pool_capacity([p], 1))
    with pytest.raises(MOCError):                 # no linear-source pool
        flat_only.submit(p, linear_source=True)
    with pytest.raises(MOCError):                 # moments of a flat solve
        flat_only.submit(p, fixed_source_moments=np.zeros((p.num_fsrs, 3, 7)))
    flat_only.close()
    srv = _ls_server([p], 1)
    bad = dict(p.linear_source)
    bad["ang_dir"] = 2.0 * np.asarray(bad["ang_dir"])   # not unit vectors
    with pytest.raises(MOCError):
        srv.submit(p, linear_source=bad)
    bad = dict(p.linear_source)
    bad["seg_x"] = np.array(bad["seg_x"], np.float32)
    bad["seg_x"][3] = np.nan
    with pytest.raises(MOCError):
        srv.submit(p, linear_source=bad)
    with pytest.raises(MOCError):                 # a flat request, no flat pool
        srv.submit(p)
    # 6 group pairs per lane: a flat-source shape, above the linear source's 5
    srv.add_pool(96, 3, 1, 1, 1, 10, 10, 10, shape=(8, 6, EXP_INTRINSIC))
    with pytest.raises(MOCError):
        srv.add_pool(96, 3, 1, 1, 1, 10, 10, 10, shape=(8, 6, EXP_INTRINSIC),
                     linear_source=True)
    srv.close()
