"""Shading server on the GPU: every request's result is the same served
alone, served in a mix of concurrent requests, and computed by the plain
per-request executor; admission never exceeds the HBM budget and
requests larger than a wave or than free memory still complete."""
import threading

import numpy as np
import pytest

from helpers import float_equal, og

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from openshadinglanguage_gb300 import serving, workloads  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


@pytest.fixture(scope="module")
def setup():
    ss = og.ShadingSystem()
    specs = workloads.c3_specs()
    groups = [workloads.c3_group(ss, name, oso) for (name, oso, n, t) in specs[:12]]
    reqs = serving.make_requests(torch, groups, 40, seed=7, lo=100, hi=40000)
    # the plain executor per request gives the reference outputs
    for r in reqs:
        dP = r.P.cuda()
        o = torch.zeros(r.n * 4, device="cuda")
        ss.execute_batch(r.group, r.n, og.make_globals(P=dP), 0, o.data_ptr(), sync=True)
        r.ref = o.cpu().numpy()
    return ss, groups, reqs


def outputs_equal(reqs):
    for i, r in enumerate(reqs):
        got = r.out.numpy()
        assert np.all(float_equal(got, r.ref)), "request %d (group %d, %d points)" % (i, r.k, r.n)


def test_alone_equals_plain(setup):
    ss, groups, reqs = setup
    srv = ss.server(budget_bytes=1 << 30, streams=2)
    for r in reqs:
        r.out.zero_()
        st = srv.wait(srv.submit(r.group, r.n, r.G, r.out))
        assert st["done_ns"] >= st["admit_ns"] >= st["submit_ns"] > 0
    outputs_equal(reqs)
    s = srv.stats()
    assert s["completed"] == len(reqs) and s["failed"] == 0
    srv.close()


def test_mix_equals_alone(setup):
    ss, groups, reqs = setup
    srv = ss.server(budget_bytes=1 << 30, streams=3, max_wave_points=60000)
    for r in reqs:
        r.out.zero_()
    tickets = [srv.submit(r.group, r.n, r.G, r.out) for r in reqs]
    stats = [srv.wait(t) for t in tickets]
    outputs_equal(reqs)
    s = srv.stats()
    assert s["waves"] > 1  # requests shared waves and waves overlapped
    assert len({st["wave"] for st in stats}) < len(reqs)
    assert ss.device_status() == 0
    srv.close()


def test_concurrent_submitters_and_small_budget(setup):
    ss, groups, reqs = setup
    # an arena that holds only a few requests at a time: admission waits for memory
    srv = ss.server(budget_bytes=(1 << 30), streams=2, block=256, max_wave_points=20000, arena_bytes=3 << 20)
    cap = srv.stats()["arena_capacity"]
    for r in reqs:
        r.out.zero_()

    def submit_some(part):
        ts = [srv.submit(r.group, r.n, r.G, r.out) for r in part]
        for t in ts:
            srv.wait(t)

    parts = [reqs[i::4] for i in range(4)]
    ths = [threading.Thread(target=submit_some, args=(p,)) for p in parts]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    outputs_equal(reqs)
    s = srv.stats()
    assert s["completed"] == len(reqs) and s["arena_high_water"] <= cap
    assert s["waves"] >= sum(r.n for r in reqs) * 28 // cap  # memory, not the wave limit, paced admission
    srv.close()


def test_request_larger_than_budget_is_refused(setup):
    ss, groups, reqs = setup
    srv = ss.server(budget_bytes=(1 << 30), streams=1, block=256, arena_bytes=8 << 20)
    cap = srv.stats()["arena_capacity"]
    n = cap // 16 + 1024  # inputs + outputs exceed the arena
    out = np.zeros(4, np.float32)
    P = np.zeros((3, 1), np.float32)
    G = og.make_globals(P=P)
    with pytest.raises(og.OSLError):
        srv.submit(groups[0], n, G, out.ctypes.data, n * 16)
    srv.close()


def test_open_loop_poisson_run(setup):
    ss, groups, reqs = setup
    srv = ss.server(budget_bytes=1 << 30, streams=3)
    for g in groups:
        srv.register(g)
    res = serving.run_server(srv, reqs, rate_rps=2000.0)
    assert res["requests"] == len(reqs) and res["p99_ms"] >= res["p50_ms"] > 0
    outputs_equal(reqs)
    srv.close()
    base = serving.run_plain(torch, ss, reqs, rate_rps=2000.0)
    assert base["requests"] == len(reqs)
    outputs_equal(reqs)


def test_failed_request_fails_alone_in_a_mixed_wave(setup):
    """A request whose kernel raises a status bit (here the loop limit) fails
    with that status; the requests that shared its wave complete with their
    plain-executor results, and no bit is left for a later call to find."""
    from test_loop_limit import W, H, two_loops
    from helpers import pixel_grid
    ss, groups, reqs = setup
    ss.attribute("max_loop_iterations", 5)
    ss.LoadMemoryCompiledShader("two_loops_srv", two_loops(100).replace("two_loops", "two_loops_srv"))
    lg = ss.ShaderGroupBegin("two_loops_srv_group")
    ss.Shader(lg, "surface", "two_loops_srv", "layer1")
    ss.ShaderGroupEnd(lg)
    ss.add_symlocs(lg, [og.SymLocationDesc("count", og.TypeInt, False, og.SymArenaOutputs, 0, 4)])
    ss.optimize_group(lg)  # lowered with the limit of 5 back edges per point
    ss.attribute("max_loop_iterations", 0)
    u, _ = pixel_grid(W, H)
    lu = torch.from_numpy(u).pin_memory()
    lout = torch.zeros(W * H, dtype=torch.int32).pin_memory()
    srv = ss.server(budget_bytes=1 << 30, streams=1, max_wave_points=1 << 24)
    part = reqs[:6]
    for r in part:
        r.out.zero_()
    tickets = [srv.submit(r.group, r.n, r.G, r.out) for r in part[:3]]
    bad = srv.submit(lg, W * H, og.make_globals(u=lu), lout)
    tickets += [srv.submit(r.group, r.n, r.G, r.out) for r in part[3:]]
    with pytest.raises(og.OSLError, match="status bits 8"):
        srv.wait(bad)
    stats = [srv.wait(t) for t in tickets]
    assert all(st["status"] == 0 for st in stats)
    outputs_equal(part)
    s = srv.stats()
    assert s["failed"] == 1 and s["completed"] == len(part)
    srv.close()
    assert ss.device_status() == 0


def test_jit_server_equals_plain(setup):
    """With the system attribute "jit", waves run one kernel specialized to
    the resident programs: the same outputs as the plain interpreter."""
    ss, groups, reqs = setup
    ssj = og.ShadingSystem()
    ssj.attribute("jit", 1)
    specs = workloads.c3_specs()
    jgroups = [workloads.c3_group(ssj, name, oso) for (name, oso, n, t) in specs[:12]]
    jreqs = serving.make_requests(torch, jgroups, 40, seed=7, lo=100, hi=40000)
    srv = ssj.server(budget_bytes=1 << 30, streams=3, max_wave_points=60000)
    for g in jgroups:
        srv.register(g)
    tickets = [srv.submit(r.group, r.n, r.G, r.out) for r in jreqs]
    for t in tickets:
        srv.wait(t)
    for i, (r, ref) in enumerate(zip(jreqs, reqs)):
        assert np.all(float_equal(r.out.numpy(), ref.ref)), "request %d" % i
    assert srv.stats()["failed"] == 0 and ssj.device_status() == 0
    srv.close()
