"""The batched solve server (include/openmoc_gb300_serve.h) on the GPU.

Each batched result must match OpenMOC's own on the fixtures (keff within
1e-5, fluxes within 1e-4 relative, the parity bar) and the plain one-solve
GB300Solver on generated problems, and a request must give the same result
alone and in a mix of other requests (within the same tolerances; tally
atomics make the last bits order-dependent).

Two solves stopped by the source criterion can stop one iteration apart
(the tally atomics decide which side of the threshold a residual falls),
and near that point one iteration of a pin cell's slowly converging
upscatter groups still moves the flux by about 2e-4 (the FP64 oracle moves
keff by 3e-5 between the 1e-5 stop at 39 iterations and 1e-8 at 56).
Comparisons of generated problems therefore run both sides for the same
FIXED_ITERS iterations (a threshold no solve reaches), where only the order
of the atomics differs.
"""
import time

import numpy as np
import pytest

from conftest import CASES, CASES_3D, load_case
from openmoc_gb300 import GB300Solver, lattice
from openmoc_gb300._native import MOCError
from openmoc_gb300.serving import Server, pool_capacity
from openmoc_gb300.solver import EXP_INTRINSIC

pytestmark = pytest.mark.gpu

KEFF_TOL = 1e-5
FLUX_TOL = 1e-4
FIXED_ITERS = 60
NEVER = 1e-12   # threshold: stop at FIXED_ITERS


def max_rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.max(np.abs(a - b) / np.abs(b)))


# Sweep shapes (lanes per track direction, group pairs per lane) with the
# hardware-ex2 evaluator: a pool and a single solver given the same
# evaluator differ only in the order of the tally atomics.
SHAPES = {2: (1, 1), 7: (4, 1), 16: (8, 1), 70: (8, 5), 80: (8, 5)}


def make_server(problems, max_solves, k=8, graphs=True, fixed_shape=True):
    srv = Server(iterations_per_poll=k, use_graphs=graphs)
    by_key = {}
    for p in problems:
        by_key.setdefault((p.num_groups, p.num_polar_half), []).append(p)
    for (G, ph), ps in sorted(by_key.items()):
        shape = (*SHAPES[G], EXP_INTRINSIC) if fixed_shape else None
        srv.add_pool(G, ph, shape=shape, **pool_capacity(ps, max_solves))
    return srv


def single(p, kind="eigenvalue", max_iters=FIXED_ITERS, res_type=1, k_eff=1.0,
           threshold=NEVER):
    s = GB300Solver(p)
    s.setConvergenceThreshold(threshold)
    s.useExponentialIntrinsic()
    s.setSweepShape(*SHAPES[p.num_groups])
    if kind == "eigenvalue":
        s.computeEigenvalue(max_iters, res_type)
    else:
        s.computeSource(max_iters, k_eff, res_type)
    out = dict(keff=s.getKeff(), flux=s.getFluxes(), iterations=s.getNumIterations())
    s.close()
    return out


def test_fixtures_batched_match_openmoc():
    cases = {c: load_case(c) for c in CASES + CASES_3D}
    # pools autotune their sweep shape and evaluator on the first batch
    srv = make_server([v[0] for v in cases.values()], 2, fixed_shape=False)
    tickets = {}
    for c, (p, sc, _) in cases.items():
        tickets[c] = srv.submit(p, "eigenvalue", int(sc["max_iters"]),
                                int(sc["res_type"]), threshold=sc["tolerance"])
    srv.run_until_idle()
    for c, (p, sc, arr) in cases.items():
        r = srv.wait(tickets[c], timeout=0)
        _, sc64, arr64 = load_case(c, "f64")
        assert r["converged"]
        assert abs(r["iterations"] - int(sc["iterations"])) <= 2, c
        assert abs(r["keff"] - sc["keff"]) <= KEFF_TOL, (c, r["keff"], sc["keff"])
        assert max_rel(r["flux"], arr["flux"]) <= FLUX_TOL, c
        assert abs(r["keff"] - sc64["keff"]) <= 1.5 * KEFF_TOL, c
        assert max_rel(r["flux"], arr64["flux"]) <= FLUX_TOL, c
    st = srv.stats()
    assert st["completed"] == len(cases) and st["failed"] == 0
    assert st["graph_captures"] >= 1
    srv.close()


def mix(n_extra=6):
    """A mix of uneven generated problems (pin cells and small lattices,
    7 groups, perturbed cross sections)."""
    ps = [lattice.pin_cell(7, 16 + 4 * (i % 3), 0.08, config=0, perturb=(100 + i, 0.05))
          for i in range(n_extra // 2)]
    ps += [lattice.square_lattice(3, 7, 16, 0.1, config=2, perturb=(200 + i, 0.05))
           for i in range(n_extra - n_extra // 2)]
    return ps


def test_same_result_alone_and_in_the_mix():
    target = lattice.square_lattice(3, 7, 24, 0.08, config=3, perturb=(7, 0.05))
    others = mix(6)
    alone = make_server([target] + others, 8)
    ta = alone.submit(target, max_iters=FIXED_ITERS, threshold=NEVER)
    alone.run_until_idle()
    ra = alone.wait(ta, timeout=0)
    alone.close()

    crowd = make_server([target] + others, 8)
    first = [crowd.submit(p) for p in others[:3]]
    crowd.step()                       # others already running ...
    tb = crowd.submit(target, max_iters=FIXED_ITERS,
                      threshold=NEVER)   # ... when the target arrives
    rest = [crowd.submit(p) for p in others[3:]]
    crowd.run_until_idle()
    rb = crowd.wait(tb, timeout=0)
    for t in first + rest:
        assert crowd.wait(t, timeout=0)["converged"]
    crowd.close()

    ref = single(target)
    for r in (ra, rb):
        assert r["iterations"] == ref["iterations"] == FIXED_ITERS
        assert abs(r["keff"] - ref["keff"]) <= KEFF_TOL
        assert max_rel(r["flux"], ref["flux"]) <= FLUX_TOL
    assert abs(ra["keff"] - rb["keff"]) <= KEFF_TOL
    assert max_rel(ra["flux"], rb["flux"]) <= FLUX_TOL


def test_continuous_admission_with_two_slots():
    ps = mix(6)
    srv = make_server(ps, 2, k=4)
    tickets = [srv.submit(p, max_iters=FIXED_ITERS, threshold=NEVER) for p in ps]
    n_pending = srv.step()
    assert n_pending == len(ps)         # two admitted, four queued
    srv.run_until_idle()
    for p, t in zip(ps, tickets):
        r = srv.wait(t, timeout=0)
        ref = single(p)
        assert r["iterations"] == ref["iterations"] == FIXED_ITERS
        assert abs(r["keff"] - ref["keff"]) <= KEFF_TOL
        assert max_rel(r["flux"], ref["flux"]) <= FLUX_TOL
    st = srv.stats()
    assert st["admitted"] == len(ps) and st["completed"] == len(ps)
    assert st["graph_captures"] >= 3    # the set of live solves changed
    srv.close()


def test_wide_pool_with_many_materials_runs_from_graphs():
    """A 70-group pool holding 56 pin cells at once (112 material rows): the
    sweep's cross-section table and source ring then take more than 48 KB of
    dynamic shared memory, and the sweep runs from captured graphs (the shape
    is fixed, so no autotuning launch precedes the first capture); the
    request loop reports no error and the solves match the single solver."""
    base = lattice.pin_cell(70, 8, 0.1)
    ps = [base.with_xs(*lattice.pack_materials(
              lattice._fuel_mod(0, 70, 1, perturb=(2000 + i, 0.05)))) for i in range(56)]
    srv = make_server(ps, 56, k=4)
    tickets = [srv.submit(p, max_iters=8, threshold=NEVER) for p in ps]
    srv.run_until_idle()
    res = [srv.wait(t, timeout=0) for t in tickets]
    assert srv.loop_error() == ""
    assert all(r["iterations"] == 8 for r in res)
    assert srv.stats()["graph_captures"] >= 1
    for i in (0, 55):
        ref = single(ps[i], max_iters=8)
        assert abs(res[i]["keff"] - ref["keff"]) <= 2e-6 * ref["keff"]
        assert max_rel(res[i]["flux"], ref["flux"]) <= 2e-5
    srv.close()


def test_pools_sharing_a_sweep_instance_replay_their_graphs():
    """A 70-group and an 80-group pool sweep with the same kernel instance
    (8 lanes x 5 group pairs) and need different shared memory for it
    (112 and 90 material rows: about 52 and 49 KB); each replays its
    captured graph between the other's blocks, and every solve matches the
    single solver."""
    def pins(G, n, seed):
        base = lattice.pin_cell(G, 8, 0.1)
        return [base.with_xs(*lattice.pack_materials(
                    lattice._fuel_mod(0, G, 1, perturb=(seed + i, 0.05)))) for i in range(n)]
    ps = pins(70, 56, 3000) + pins(80, 45, 4000)
    srv = make_server(ps, 56, k=4)
    tickets = [srv.submit(p, max_iters=12, threshold=NEVER) for p in ps]
    srv.run_until_idle()
    res = [srv.wait(t, timeout=0) for t in tickets]
    assert srv.loop_error() == ""
    assert all(r["iterations"] == 12 for r in res)
    for i in (0, 56):
        ref = single(ps[i], max_iters=12)
        assert abs(res[i]["keff"] - ref["keff"]) <= 2e-6 * ref["keff"]
        assert max_rel(res[i]["flux"], ref["flux"]) <= 2e-5
    srv.close()


def test_unconverged_iterates_match_the_single_solver():
    """Six iterations, far from convergence: every iterate of a solve that
    reuses a freed slot must equal the single solver's to rounding, which
    checks the starting state and the per-solve reductions directly."""
    ps = mix(6)
    srv = make_server(ps, 2, k=4)
    tickets = [srv.submit(p, max_iters=6, threshold=NEVER) for p in ps]
    srv.run_until_idle()
    for p, t in zip(ps, tickets):
        r = srv.wait(t, timeout=0)
        ref = single(p, max_iters=6)
        assert r["iterations"] == ref["iterations"] == 6
        assert abs(r["keff"] - ref["keff"]) <= 2e-6 * ref["keff"]
        assert max_rel(r["flux"], ref["flux"]) <= 2e-5
    srv.close()


def test_fixed_source_requests():
    p = lattice.square_lattice(3, 7, 16, 0.1, config=4)
    q = np.zeros((p.num_fsrs, p.num_groups), np.float32)
    fuel = np.nonzero(p.fsr_mat == 0)[0]
    q[fuel, :] = 1.0
    k_sub = 1.5   # above the lattice's own keff: a convergent source problem
    srv = make_server([p], 4)
    t1 = srv.submit(p, "source", FIXED_ITERS, 2, k_eff=k_sub, fixed_source=q,
                    threshold=NEVER)
    t2 = srv.submit(p, "eigenvalue", FIXED_ITERS, threshold=NEVER)
    srv.run_until_idle()
    r1 = srv.wait(t1, timeout=0)
    r2 = srv.wait(t2, timeout=0)
    srv.close()

    s = GB300Solver(p)
    s.setConvergenceThreshold(NEVER)
    s.useExponentialIntrinsic()
    s.setSweepShape(*SHAPES[p.num_groups])
    for f in fuel:
        for g in range(p.num_groups):
            s.setFixedSourceByFSR(int(f), g + 1, 1.0)
    s.computeSource(FIXED_ITERS, k_sub, 2)
    ref_flux = s.getFluxes()
    ref_iters = s.getNumIterations()
    s.close()
    assert r1["keff"] == pytest.approx(k_sub)
    assert max_rel(r1["flux"], ref_flux) <= FLUX_TOL
    assert r1["iterations"] == ref_iters == FIXED_ITERS
    ref2 = single(p)
    assert abs(r2["keff"] - ref2["keff"]) <= KEFF_TOL
    assert max_rel(r2["flux"], ref2["flux"]) <= FLUX_TOL


def test_loop_thread_and_graph_free_mode_agree():
    ps = mix(4)
    srv = make_server(ps, 4, k=8, graphs=True)
    srv.start()
    tickets = []
    for p in ps:
        tickets.append(srv.submit(p, max_iters=FIXED_ITERS, threshold=NEVER))
        time.sleep(0.002)
    res = [srv.wait(t, timeout=120) for t in tickets]
    srv.stop()
    assert sorted(srv.poll()) == sorted(tickets)
    srv.close()

    plain = make_server(ps, 4, k=8, graphs=False)
    t2 = [plain.submit(p, max_iters=FIXED_ITERS, threshold=NEVER) for p in ps]
    plain.run_until_idle()
    for r, t in zip(res, t2):
        r2 = plain.wait(t, timeout=0)
        assert abs(r["keff"] - r2["keff"]) <= KEFF_TOL
        assert max_rel(r["flux"], r2["flux"]) <= FLUX_TOL
        assert r["t_submit"] <= r["t_admit"] <= r["t_done"]
    plain.close()


def test_bad_request_is_refused_on_submit():
    p = lattice.pin_cell(7, 16, 0.1)
    srv = make_server([p], 1)
    with pytest.raises(MOCError, match="threshold"):
        srv.submit(p, "eigenvalue", threshold=-1.0)
    with pytest.raises(MOCError, match="no flat-source pool"):
        srv.submit(lattice.pin_cell(2, 16, 0.1))     # no pool for 2 groups
    big = lattice.square_lattice(3, 7, 16, 0.1, config=0)
    with pytest.raises(MOCError, match="capacity"):
        srv.submit(big)
    assert srv.stats()["submitted"] == 0
    srv.close()


def test_fixed_source_fixture_through_a_pool():
    """OpenMOC's computeSource fixture, solved in a pool beside eigenvalue
    solves, against OpenMOC's FP32 and FP64 results."""
    p, sc, arr = load_case("src3_g7")
    _, _, arr64 = load_case("src3_g7", "f64")
    others = mix(4)
    srv = make_server([p] + others, 8, fixed_shape=False)
    ts = [srv.submit(q) for q in others[:2]]
    t = srv.submit(p, "source", int(sc["max_iters"]), int(sc["res_type"]),
                   k_eff=sc["k_source"], threshold=sc["tolerance"])
    ts += [srv.submit(q) for q in others[2:]]
    srv.run_until_idle()
    r = srv.wait(t, timeout=0)
    for x in ts:
        assert srv.wait(x, timeout=0)["converged"]
    srv.close()
    assert r["converged"]
    assert abs(r["iterations"] - int(sc["iterations"])) <= 1
    assert r["keff"] == pytest.approx(sc["k_source"])
    assert max_rel(r["flux"], arr["flux"]) <= FLUX_TOL
    assert max_rel(r["flux"], arr64["flux"]) <= FLUX_TOL


def test_fixed_flux_fixture_through_a_pool():
    """OpenMOC's computeFlux fixture (the fixed source alone, computed once
    from a zero flux; SCALAR_FLUX residual) solved in a pool beside
    eigenvalue and computeSource solves, against OpenMOC's FP32 and FP64
    results, and the same request alone against the single-problem solver."""
    p, sc, arr = load_case("flux3_g7")
    _, _, arr64 = load_case("flux3_g7", "f64")
    ps, _, _ = load_case("src3_g7")
    others = mix(4)
    srv = make_server([p, ps] + others, 8, fixed_shape=False)
    ts = [srv.submit(q) for q in others[:2]]
    t = srv.submit(p, "flux", int(sc["max_iters"]), threshold=sc["tolerance"])
    ts.append(srv.submit(ps, "source", 1000, 2, k_eff=1.0, threshold=1e-5))
    ts += [srv.submit(q) for q in others[2:]]
    srv.run_until_idle()
    r = srv.wait(t, timeout=0)
    for x in ts:
        assert srv.wait(x, timeout=0)["converged"]
    srv.close()
    assert r["converged"]
    assert abs(r["iterations"] - int(sc["iterations"])) <= 1
    assert max_rel(r["flux"], arr["flux"]) <= FLUX_TOL
    assert max_rel(r["flux"], arr64["flux"]) <= FLUX_TOL
    s = GB300Solver(p)
    s.setConvergenceThreshold(sc["tolerance"])
    s.computeFlux(int(sc["max_iters"]), True)
    assert r["iterations"] == s.getNumIterations()
    assert max_rel(r["flux"], s.getFluxes()) <= 1e-5
    s.close()
