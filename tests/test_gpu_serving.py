"""Continuous-batching server: every job's result is the same alone, in a mix
and from the plain per-job solver (max |d eta| <= 1e-4; alone vs in a mix
bit-identical), admission respects the HBM budget, and graph replay equals
eager launches."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

ETA_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _built():
    from jax_am_gb300 import _build
    _build.build()


def make_job(shape, n, steps, seed, grad=1e6, arrival=0.0, aniso=0.0):
    from jax_am_gb300.phase_field.allen_cahn import PFSolver, Quench
    from jax_am_gb300.phase_field.utils import Field
    from jax_am_gb300.serving import Job
    nx, ny, nz = shape
    pf_args = dict(Nx=nx, Ny=ny, Nz=nz, h=1e-6, num_grains=max(2, nx * ny * nz // 500),
                   num_oris=n, T_liquidus=1700.0, gas_const=8.3, Qg=1.4e5, L0=3.5e3,
                   kappa_g=2.77e-6, m_g=2.4e5, anisotropy=aniso, ad_hoc=1.0,
                   force_liquid_zero=True, liquid_shift=1.0)
    poly = Field(pf_args, seed=seed)
    dt = PFSolver(pf_args, poly).stable_dt()
    q = Quench(1700.0, grad, 0.1, z0=0.5 * nz * 1e-6)
    return Job(pf_args, poly, q, steps, float(np.float32(dt)), arrival=arrival)


def _mix():
    return [make_job((40, 33, 17), 10, 37, 1), make_job((24, 31, 9), 12, 50, 2, aniso=0.15),
            make_job((17, 16, 21), 7, 23, 3), make_job((33, 9, 16), 20, 41, 4, grad=5e5),
            make_job((13, 11, 5), 3, 29, 5)]  # N*n odd: buffer sizes not a multiple of 16 B


def test_batch_matches_plain_solver_and_mix_equals_alone():
    from jax_am_gb300 import _lib
    from jax_am_gb300.serving import BatchServer, run_sequential
    mix = _mix()
    srv = BatchServer(max_jobs=8, graph_steps=8)
    for j in mix:
        srv.submit(j)
    srv.run(realtime=False)
    plain = _mix()
    run_sequential(plain, realtime=False)
    for jb, jp in zip(mix, plain):
        err = (jb.result - jp.result).abs().max().item()
        print(f"job {jb.id}: cells={jb.cells} n={jb.num_oris} steps={jb.steps}: "
              f"max |d eta| batch vs plain = {err:.3e}")
        assert err <= ETA_TOL
    # the same job alone: bit-identical to its result in the mix
    alone = make_job((24, 31, 9), 12, 50, 2, aniso=0.15)
    srv2 = BatchServer(max_jobs=8, graph_steps=8)
    srv2.submit(alone)
    srv2.run(realtime=False)
    assert torch.equal(alone.result, mix[1].result)
    assert _lib.device_error() == 0


@pytest.mark.parametrize("pad", [True, False], ids=["padded_tma_body", "unpadded_warp_body"])
def test_batch_bodies_match_plain_solver(pad):
    """Orientation counts padded to a multiple of 4 run the TMA-fed unit
    body (persistent CTAs re-initialise its barriers for every unit);
    unpadded odd counts run the warp-per-cells body; both match the plain
    per-job solver, and a CTA can take units of both bodies in turn."""
    from jax_am_gb300 import _lib
    from jax_am_gb300.serving import BatchServer, run_sequential
    mix = _mix() + [make_job((36, 20, 12), 16, 33, 6, aniso=0.15)]
    srv = BatchServer(max_jobs=8, graph_steps=8, pad_oris=pad)
    for j in mix:
        srv.submit(j)
    srv.run(realtime=False)
    plain = _mix() + [make_job((36, 20, 12), 16, 33, 6, aniso=0.15)]
    run_sequential(plain, realtime=False)
    for jb, jp in zip(mix, plain):
        err = (jb.result - jp.result).abs().max().item()
        assert err <= ETA_TOL, (jb.cells, jb.num_oris, err)
    assert _lib.device_error() == 0


def test_graph_replay_equals_eager():
    from jax_am_gb300.serving import BatchServer
    res = []
    for use_graph in (False, True):
        jobs = _mix()
        srv = BatchServer(max_jobs=8, graph_steps=4)
        for j in jobs:
            srv.submit(j)
        srv.run(use_graph=use_graph, realtime=False)
        res.append([j.result for j in jobs])
    for a, b in zip(*res):
        assert torch.equal(a, b)


def test_hbm_budget_limits_admission():
    from jax_am_gb300.serving import BatchServer
    jobs = _mix()
    budget = max(j.nbytes for j in jobs) * 1.5  # never two of the big ones together
    srv = BatchServer(hbm_budget=budget, max_jobs=8, graph_steps=8)
    for j in jobs:
        srv.submit(j)
    out = srv.run(realtime=False)
    assert out["jobs"] == len(jobs)
    assert srv.peak_bytes <= budget
    ref = _mix()
    srv2 = BatchServer(max_jobs=8, graph_steps=8)
    for j in ref:
        srv2.submit(j)
    srv2.run(realtime=False)
    for a, b in zip(jobs, ref):
        assert torch.equal(a.result, b.result)
    with pytest.raises(ValueError):
        BatchServer(hbm_budget=1000).submit(make_job((8, 8, 8), 4, 5, 9))


def test_realtime_arrivals_are_admitted_while_others_run():
    from jax_am_gb300.serving import BatchServer
    jobs = [make_job((48, 48, 24), 10, 400, 11, arrival=0.0),
            make_job((20, 20, 10), 8, 60, 12, arrival=0.05),
            make_job((20, 20, 10), 8, 60, 13, arrival=0.10)]
    srv = BatchServer(max_jobs=4, graph_steps=8)
    for j in jobs:
        srv.submit(j)
    out = srv.run(realtime=True)
    assert out["jobs"] == 3
    for j in jobs:
        assert j.finished >= j.arrival and j.admitted >= j.arrival
    print(out)


def test_resident_sequential_baseline_matches_stepper():
    """The graph-replayed per-job baseline (QuenchRun) gives the per-step
    stepper's results (the same kernels, launched from a graph)."""
    from jax_am_gb300.serving import run_sequential, run_sequential_resident
    a, b = _mix(), _mix()
    ra = run_sequential(a, realtime=False)
    rb = run_sequential_resident(b, realtime=False)
    assert ra["jobs"] == rb["jobs"] == len(a)
    for ja, jb in zip(a, b):
        assert torch.equal(ja.result, jb.result), (ja.cells, ja.num_oris, ja.steps)

