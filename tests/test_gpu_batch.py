"""Persistent batch executor on the GPU: one launch over many different
groups gives the same bits as one plain launch per group (and as the
oracle), with and without CUDA-graph replay and after autotuning."""
import numpy as np
import pytest

from helpers import float_equal, og, oracle_run

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from openshadinglanguage_gb300 import workloads  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


class Req:
    pass


def c3_requests(ss, scale=32, groups=None):
    reqs = []
    for k, (name, oso, npts, target) in enumerate(workloads.c3_specs()):
        if groups is not None and k not in groups:
            continue
        r = Req()
        r.k, r.name = k, name
        r.g = workloads.c3_group(ss, name, oso)
        r.n = max(67, npts // scale)  # ragged: rarely a multiple of the block
        r.hP = workloads.c3_points(k, r.n)
        r.dP = torch.from_numpy(r.hP).cuda()
        r.G = og.make_globals(P=r.dP)
        r.rec = workloads.C3_REC
        reqs.append(r)
    return reqs


def outputs(reqs):
    return [torch.full((r.n * r.rec,), -7.0, dtype=torch.float32, device="cuda") for r in reqs]


def same(a, b):
    return bool(np.all(float_equal(a, b)))


def run_plain(ss, reqs):
    outs = outputs(reqs)
    st = torch.cuda.current_stream().cuda_stream
    for r, o in zip(reqs, outs):
        ss.execute_batch(r.g, r.n, r.G, 0, o.data_ptr(), st)
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in outs]


def run_batch(ss, reqs, use_graph, block=256, heap=-1, times=1, tune=False, ppt=1):
    outs = outputs(reqs)
    b = ss.batch()
    for r, o in zip(reqs, outs):
        b.add(r.g, r.n, r.G, 0, o.data_ptr())
    b.set_launch(block=block, heap_smem=heap, use_graph=use_graph, points_per_thread=ppt)
    st = torch.cuda.current_stream().cuda_stream
    tuned = None
    if tune:
        tuned = b.autotune(st, reps=1)
        for o in outs:
            o.fill_(-7.0)
    for _ in range(times):
        b.execute(st)
    torch.cuda.synchronize()
    res = [o.cpu().numpy() for o in outs]
    launch = b.last_launch()
    b.close()
    return res, launch, tuned


@pytest.fixture(scope="module")
def c3():
    ss = og.ShadingSystem()
    reqs = c3_requests(ss)
    plain = run_plain(ss, reqs)
    assert ss.device_status() == 0
    return ss, reqs, plain


def test_plain_matches_oracle(c3):
    ss, reqs, plain = c3
    for r, p in zip(reqs, plain):
        ref = np.zeros((r.n, r.rec), np.float32)
        assert oracle_run(r.g.program_bytes(), r.n, og.make_globals(P=r.hP), ref) == 0
        assert same(p.reshape(r.n, r.rec), ref), r.name


@pytest.mark.parametrize("block,heap,ppt", [(256, -1, 1), (128, 1, 1), (512, 0, 1), (256, 0, 2), (32, 1, 4),
                                            (512, 0, 4), (64, 1, 2)])
def test_persistent_batch_matches_plain(c3, block, heap, ppt):
    ss, reqs, plain = c3
    got, launch, _ = run_batch(ss, reqs, use_graph=False, block=block, heap=heap, ppt=ppt)
    assert launch["block"] == block and launch["points_per_thread"] == ppt
    if heap >= 0:
        assert launch["heap_smem"] == heap
    for r, a, b in zip(reqs, got, plain):
        assert same(a, b), r.name
    assert ss.device_status() == 0


def test_graph_replay_matches_plain(c3):
    ss, reqs, plain = c3
    got, _, _ = run_batch(ss, reqs, use_graph=True, times=3)
    for r, a, b in zip(reqs, got, plain):
        assert same(a, b), r.name


def test_autotuned_batch_matches_plain(c3):
    ss, reqs, plain = c3
    got, launch, (best, cands) = run_batch(ss, reqs, use_graph=True, tune=True)
    assert len(cands) >= 9
    assert {c["points_per_thread"] for c in cands} == {1, 2, 4}
    assert best["ms"] == min(c["ms"] for c in cands)
    assert launch["block"] == best["block"] and launch["heap_smem"] == best["heap_smem"]
    for r, a, b in zip(reqs, got, plain):
        assert same(a, b), r.name


def test_jit_batch_matches_plain(c3):
    """A batch created with the system attribute "jit" runs one persistent
    kernel specialized to its programs: same bits as the plain interpreter
    launches, with graph replay and after its (block size) autotune."""
    ss, reqs, plain = c3
    pick = list(range(0, len(reqs), 6))
    ssj = og.ShadingSystem()
    ssj.attribute("jit", 1)
    jreqs = c3_requests(ssj, groups={reqs[i].k for i in pick})
    got, launch, (best, cands) = run_batch(ssj, jreqs, use_graph=True, tune=True, times=2)
    assert {c["block"] for c in cands} <= {128, 256} and len(cands) >= 1
    assert launch["points_per_thread"] == 1
    for i, r, a in zip(pick, jreqs, got):
        assert same(a, plain[i]), r.name
    assert ssj.device_status() == 0


def test_batch_with_closure_group_and_empty_requests():
    ss = og.ShadingSystem()
    reqs = c3_requests(ss, scale=256, groups={1, 9, 30})
    W = H = 64
    g2 = workloads.c2_group(ss)
    u, v, I = workloads.c2_inputs(W, H)
    du, dv, dI = (torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (u, v, I))
    G2 = workloads.c2_globals(og.make_globals, du, dv, dI)
    rec2 = workloads.C2_STRIDE // 4
    st = torch.cuda.current_stream().cuda_stream
    o2p = torch.zeros(W * H * rec2, device="cuda")
    ss.execute_batch(g2, W * H, G2, 0, o2p.data_ptr(), st)
    plain = run_plain(ss, reqs)
    outs = outputs(reqs)
    o2b = torch.zeros(W * H * rec2, device="cuda")
    b = ss.batch()
    b.execute(st)  # empty batch: nothing to do
    for r, o in zip(reqs, outs):
        b.add(r.g, r.n, r.G, 0, o.data_ptr())
    b.add(reqs[0].g, 0, reqs[0].G, 0, 0)  # zero-point request is dropped
    b.add(g2, W * H, G2, 0, o2b.data_ptr())
    b.execute(st)
    torch.cuda.synchronize()
    assert ss.device_status() == 0
    assert same(o2b.cpu().numpy(), o2p.cpu().numpy())
    for r, o, p in zip(reqs, outs, plain):
        assert same(o.cpu().numpy(), p), r.name
    b.close()


def test_jit_groups_builds_every_kernel(c3):
    """jit_groups (BatchedExecutor::jit_all_groups) builds the specialized
    kernels of several groups on worker threads; each group then runs its
    own kernel with the plain interpreter's bits."""
    ss, reqs, plain = c3
    pick = list(range(3, len(reqs), 9))
    ssj = og.ShadingSystem()
    ssj.attribute("jit", 1)
    jreqs = c3_requests(ssj, groups={reqs[i].k for i in pick})
    ssj.jit_groups([r.g for r in jreqs], nthreads=4)
    assert all(r.g.is_specialized() for r in jreqs)
    got = run_plain(ssj, jreqs)
    for i, r, a in zip(pick, jreqs, got):
        assert same(a, plain[i]), r.name
