"""The loop limit: a point that takes more loop back edges than the
program's limit (system attribute "max_loop_iterations", summed over every
loop of the group) ends with the timeout status bit. The oracle and both
device kernels count the same thing, so a shader just under the limit runs
to completion on both sides and one just over it times out on both."""
import ctypes

import numpy as np
import pytest

from helpers import float_equal, grid_globals, og, oracle_run, pixel_grid, single_layer_group
from openshadinglanguage_gb300.oso import OsoBuilder

ST_TIMEOUT = 8
W = H = 32  # u = x / (W - 1): the last column has u == 1


def two_loops(scale):
    """shader two_loops(output int count = 0)
    {
        int n = (int)(u * scale);
        int i = 0;
        while (i < n) i += 1;
        int j = 0;
        for (int k = 0; k < n; ++k) j += 2;
        count = i + j;
    }
    A point with n = (int)(u * scale) takes 2n back edges."""
    b = OsoBuilder("two_loops")
    count = b.param("int", "count", 0, output=True)
    u = b.glob("float", "u")
    n, i, j, k = (b.local("int", nm) for nm in ("n", "i", "j", "k"))
    us = b.tmp("float")
    b.op("mul", us, u, b.const("float", float(scale)))
    b.op("assign", n, us)
    b.op("assign", i, b.const("int", 0))
    c1 = b.tmp("int")
    with b.loop("while", c1) as L:
        L.cond()
        b.op("lt", c1, i, n)
        L.body()
        b.op("add", i, i, b.const("int", 1))
        L.step()
    b.op("assign", j, b.const("int", 0))
    c2 = b.tmp("int")
    with b.loop("for", c2) as L:
        b.op("assign", k, b.const("int", 0))
        L.cond()
        b.op("lt", c2, k, n)
        L.body()
        b.op("add", j, j, b.const("int", 2))
        L.step()
        b.op("add", k, k, b.const("int", 1))
    b.op("add", count, i, j)
    return b.text()


def group(limit, scale=100, jit=0):
    ss = og.ShadingSystem()
    if limit is not None:
        ss.attribute("max_loop_iterations", limit)
    if jit:
        ss.attribute("jit", 1)
    g = single_layer_group(ss, "two_loops", two_loops(scale), outputs=[
        og.SymLocationDesc("count", og.TypeInt, False, og.SymArenaOutputs, 0, 4)])
    return ss, g


def oracle_status(g):
    u, v = pixel_grid(W, H)
    out = np.zeros((W * H, 1), np.float32)
    st = oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), out)
    return st, out.view(np.int32)[:, 0]


def expected_counts(scale):
    u, _ = pixel_grid(W, H)
    n = (u * np.float32(scale)).astype(np.int32)
    return 3 * n


def test_limit_is_stored_in_the_program():
    _, g = group(200)
    blob = g.program_bytes()
    # header word 10: loop back edges per point (0 = the format's default, 2^24)
    assert int(np.frombuffer(blob[:64], np.uint32)[10]) == 200
    _, g0 = group(None)
    assert int(np.frombuffer(g0.program_bytes()[:64], np.uint32)[10]) == 0


def test_oracle_runs_to_the_limit_and_times_out_past_it():
    st, counts = oracle_status(group(200)[1])  # the widest point takes exactly 200 back edges
    assert st == 0
    assert np.array_equal(counts, expected_counts(100))
    st, _ = oracle_status(group(199)[1])
    assert st & ST_TIMEOUT
    st, _ = oracle_status(group(None)[1])  # default limit
    assert st == 0


def test_negative_limit_is_rejected():
    ss = og.ShadingSystem()
    with pytest.raises(og.OSLError):
        ss.attribute("max_loop_iterations", -1)


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
def test_device_agrees_with_the_oracle_at_the_limit(jit):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from test_gpu_parity import device_grid_globals
    u, v = pixel_grid(W, H)
    for limit, expect_timeout in ((200, False), (199, True), (1, True)):
        ss, g = group(limit, jit=jit)
        ost, ocounts = oracle_status(g)
        assert bool(ost & ST_TIMEOUT) == expect_timeout
        out = torch.zeros(W * H, dtype=torch.int32, device="cuda")
        G = device_grid_globals(u, v, W, H)
        if expect_timeout:
            with pytest.raises(og.OSLError, match="loop-iteration-limit"):
                ss.execute_batch(g, W * H, G, 0, out.data_ptr(), sync=True)
        else:
            ss.execute_batch(g, W * H, G, 0, out.data_ptr(), sync=True)
            assert np.array_equal(out.cpu().numpy(), ocounts)
        assert g.is_specialized() == bool(jit)
        # the context stays usable: the status was reported, the next launch is clean
        ss.execute_batch(g, 0, G, 0, out.data_ptr(), sync=True)
