"""The 64-group random workload and the batch API on the CPU: the
generator is deterministic and stays inside the executor's op set, every
group lowers and runs on the oracle, and the batch handle rejects bad
arguments without a GPU."""
import numpy as np
import pytest

from helpers import og, oracle_run
from openshadinglanguage_gb300 import workloads


@pytest.fixture(scope="module")
def specs():
    return workloads.c3_specs()


def test_generator_is_deterministic(specs):
    again = workloads.c3_specs()
    assert [s[1] for s in specs] == [s[1] for s in again]
    assert len(specs) == workloads.C3_GROUPS
    n = [s[2] for s in specs]
    assert min(n) >= 1000 and max(n) <= 1000000
    assert all(20 <= s[3] <= 200 for s in specs)


def test_groups_use_loops_branches_and_noise(specs):
    text = "\n".join(s[1] for s in specs)
    for word in ("\tfor\t", "\tif\t", "noise", "\"gabor\"", "\"simplex\"", "\"perlin\"", "transformn", "cellnoise"):
        assert word in text, word


def test_every_group_lowers_and_runs_on_oracle(specs):
    ss = og.ShadingSystem()
    for k, (name, oso, npts, target) in enumerate(specs):
        g = workloads.c3_group(ss, name, oso)
        blob = g.program_bytes()
        n = 256
        P = workloads.c3_points(k, n)
        out = np.zeros((n, workloads.C3_REC), np.float32)
        assert oracle_run(blob, n, og.make_globals(P=P), out) == 0, name
        assert np.count_nonzero(out) > 0, name


def test_batch_handle_on_cpu():
    ss = og.ShadingSystem()
    b = ss.batch()
    with pytest.raises(og.OSLError):
        b.set_launch(block=1024)
    b.set_launch(block=128, heap_smem=0, use_graph=False)
    b.clear()
    b.close()


def test_serving_load_generator():
    torch = pytest.importorskip("torch")
    from openshadinglanguage_gb300 import serving
    arr = serving.poisson_arrivals(1000.0, 20000, seed=3)
    gaps = np.diff(np.concatenate([[0.0], arr]))
    assert abs(gaps.mean() - 1e-3) < 5e-5 and np.all(gaps > 0)
    assert np.all(serving.poisson_arrivals(None, 5) == 0)
    groups = ["g%d" % i for i in range(64)]
    reqs = serving.make_requests(torch, groups, 50, seed=0xC4, pin=False)
    again = serving.make_requests(torch, groups, 50, seed=0xC4, pin=False)
    assert [r.n for r in reqs] == [r.n for r in again]
    assert all(256 <= r.n <= 262144 for r in reqs)
    assert all(r.P.shape == (3, r.n) and float(r.P.abs().max()) <= 10.0 for r in reqs)
