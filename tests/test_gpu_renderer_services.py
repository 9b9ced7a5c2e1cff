"""Renderer services on the GPU, interpreter and specialized kernel:
messages between layers, folded getattribute and named coordinate systems;
outputs bit-exact to the oracle and the same message-error status."""
import numpy as np
import pytest

from helpers import grid_globals, og, oracle_run, pixel_grid

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from test_gpu_parity import assert_same, dev, device_grid_globals, gpu_run  # noqa: E402
from test_messages_attributes import (attribute_group, check_attributes, check_userdata_attributes,  # noqa: E402
                                      message_group, message_testsuite_group, userdata_attribute_group,
                                      userdata_records)
from test_named_spaces import NFLOATS, check, inputs, spaces_group  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


CASES = {
    "pass": dict(),
    "derivs": dict(derivs=True),
    "mismatch": dict(recv_kw=dict(col_type="point")),
    "double": dict(send_kw=dict(double_set=True)),
    "unconnected": dict(connect=False),
}


def both(ss, g, nfloats, W=67, H=29):
    u, v = pixel_grid(W, H, centers=True)
    n = W * H
    got = gpu_run(ss, g, n, device_grid_globals(u, v, W, H, centers=True), nfloats, sync=False)
    ref = np.zeros((n, nfloats), np.float32)
    st = oracle_run(g.program_bytes(), n, grid_globals(u, v, W, H, centers=True), ref)
    return got, ref, st


@pytest.mark.parametrize("jit", [0, 1])
@pytest.mark.parametrize("case", sorted(CASES))
def test_messages_match_oracle(case, jit):
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g, stride = message_group(ss, "g%s%d" % (case, jit), **CASES[case])
    got, ref, st = both(ss, g, stride // 4)
    assert_same(got, ref)
    assert ss.device_status() == st
    if jit:
        assert g.is_specialized()


@pytest.mark.parametrize("jit", [0, 1])
@pytest.mark.parametrize("strict", [1, 0])
def test_strict_messages_match_oracle(strict, jit):
    ss = og.ShadingSystem()
    ss.attribute("strict_messages", strict)
    if jit:
        ss.attribute("jit", 1)
    extra = [("r1", og.TypeInt, 28, 4), ("r2", og.TypeInt, 32, 4), ("y", og.TypeFloat, 36, 4)]
    g, stride = message_group(ss, "st%d%d" % (strict, jit), send_kw=dict(guarded_m=True),
                              recv_kw=dict(strict_probe=True), extra=extra)
    got, ref, st = both(ss, g, stride // 4)
    assert_same(got, ref)
    assert ss.device_status() == st
    assert (st != 0) == bool(strict)


@pytest.mark.parametrize("jit", [0, 1])
def test_getattribute_matches_oracle(jit):
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = attribute_group(ss, "j%d" % jit)
    got, ref, st = both(ss, g, 17, W=33, H=5)
    assert st == 0 and ss.device_status() == 0
    assert_same(got, ref)
    check_attributes(got)


@pytest.mark.parametrize("jit", [0, 1])
def test_named_spaces_match_oracle(jit):
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = spaces_group(ss, "j%d" % jit)
    n = 5000
    P, N, T = inputs(n)
    dP, dN, dT = dev(P), dev(N), dev(T)
    got = gpu_run(ss, g, n, og.make_globals(P=dP, N=dN, dPdu=dT), NFLOATS)
    ref = np.zeros((n, NFLOATS), np.float32)
    assert oracle_run(g.program_bytes(), n, og.make_globals(P=P, N=N, dPdu=T), ref) == 0
    assert_same(got, ref)
    check(got, P, N, T)
    assert ss.device_status() == 0


@pytest.mark.parametrize("jit", [0, 1])
def test_userdata_attributes_match_oracle(jit):
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = userdata_attribute_group(ss, "j%d" % jit)
    n = 3001
    ud = userdata_records(n)
    got = gpu_run(ss, g, n, og.make_globals(u=0.5), 15, userdata=ud)
    ref = np.zeros((n, 15), np.float32)
    assert oracle_run(g.program_bytes(), n, og.make_globals(u=0.5), ref, userdata=ud) == 0
    assert_same(got, ref)
    check_userdata_attributes(got, ud)
    assert ss.device_status() == 0


@pytest.mark.parametrize("jit", [0, 1])
def test_message_testsuite_case_matches_oracle(jit):
    """color, float[4] and int messages and their error cases on the GPU"""
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g, rec = message_testsuite_group(ss)
    n = 777
    Nv = np.random.default_rng(2).normal(size=(3, n)).astype(np.float32)
    dN = dev(Nv)
    got = gpu_run(ss, g, n, og.make_globals(N=dN, u=0.25, v=0.75), rec, sync=False)
    ref = np.zeros((n, rec), np.float32)
    st = oracle_run(g.program_bytes(), n, og.make_globals(N=Nv, u=0.25, v=0.75), ref)
    assert_same(got, ref)
    assert ss.device_status() == st and st != 0
