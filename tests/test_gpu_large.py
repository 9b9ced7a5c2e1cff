"""Batches past 2^31 points: every point index, input plane offset and
output record address is 64-bit. One launch over 2^31 + 1037 points
(8.6 GB of u in, 8.6 GB of results out), interpreter and specialized
kernel; results at the int32 boundary, the tail and a random sample equal
the oracle's for the same inputs."""
import numpy as np
import pytest

from helpers import og, oracle_run, single_layer_group

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N = (1 << 31) + 1037


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    free, _ = torch.cuda.mem_get_info()
    if free < 24 << 30:
        pytest.skip("needs 24 GB of free device memory")


def shader():
    b = og.OsoBuilder("big")
    u = b.glob("float", "u")
    o = b.param("float", "o", 0.0, output=True)
    t = b.tmp("float")
    b.op("mul", t, u, u)
    b.op("add", o, t, b.const("float", 0.5))
    return b.text()


@pytest.mark.parametrize("jit", [0, 1])
def test_more_than_2_31_points(jit):
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = single_layer_group(ss, "big", shader(),
                           outputs=[og.SymLocationDesc("o", og.TypeFloat, False, og.SymArenaOutputs, 0, 4)])
    u = torch.empty(N, dtype=torch.float32, device="cuda")
    step = 1 << 28
    for s in range(0, N, step):
        e = min(N, s + step)
        u[s:e] = (torch.arange(s, e, device="cuda") % 1000003).to(torch.float32) * 1e-3
    out = torch.full((N,), -1.0, dtype=torch.float32, device="cuda")
    G = og.make_globals(u=u)
    ss.execute_batch(g, N, G, 0, out.data_ptr(), torch.cuda.current_stream().cuda_stream, sync=True)
    torch.cuda.synchronize()
    rng = np.random.default_rng(3)
    idx = np.concatenate([[0, 1, (1 << 31) - 2, (1 << 31) - 1, 1 << 31, (1 << 31) + 1, N - 2, N - 1],
                          rng.integers(0, N, 2000)]).astype(np.int64)
    ti = torch.from_numpy(idx).cuda()
    got = out[ti].cpu().numpy()
    hu = u[ti].cpu().numpy()
    ref = np.zeros((len(idx), 1), np.float32)
    assert oracle_run(g.program_bytes(), len(idx), og.make_globals(u=hu), ref) == 0
    assert np.array_equal(got.view(np.uint32), ref[:, 0].view(np.uint32))
    assert ss.device_status() == 0
    del u, out
    torch.cuda.empty_cache()
