"""Open-loop request load for the shading server and for the plain
executor launched per request: Poisson arrivals over a set of groups,
latency percentiles and throughput.

Request sizes and inputs follow the serving workload: group chosen
uniformly, point count log-uniform in [lo, hi], P uniform in [-10, 10]^3.
Latency is arrival (scheduled time) to completion (outputs in host
memory), both on the host monotonic clock, so a queue that builds up
under load shows in the percentiles.
"""
import queue
import threading
import time

import numpy as np

from .globals import make_globals


class Request:
    __slots__ = ("group", "k", "n", "P", "out", "G", "ref")


def make_requests(torch, groups, nreq, seed=0xC4, lo=256, hi=262144, rec=4, pin=True):
    """Host inputs and outputs (pinned unless pin=False) for nreq requests
    over `groups`."""
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(nreq):
        r = Request()
        r.k = int(rng.integers(len(groups)))
        r.group = groups[r.k]
        r.n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        P = rng.uniform(-10.0, 10.0, (3, r.n)).astype(np.float32)
        r.P = torch.from_numpy(P)
        r.out = torch.zeros(r.n * rec, dtype=torch.float32)
        if pin:
            r.P, r.out = r.P.pin_memory(), r.out.pin_memory()
        r.G = make_globals(P=r.P)
        reqs.append(r)
    return reqs


def poisson_arrivals(rate_rps, n, seed=0xC4A):
    """Arrival offsets (seconds) of a Poisson process with the given rate."""
    if rate_rps is None or rate_rps <= 0:
        return np.zeros(n)
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_rps, n))


def _summary(lat_ns, points, t_first, t_last):
    lat_ms = np.asarray(lat_ns, dtype=np.float64) / 1e6
    span = max(1e-9, (t_last - t_first) / 1e9)
    return {"p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
            "mean_ms": float(np.mean(lat_ms)), "throughput_mpts": points / span / 1e6, "makespan_s": span,
            "requests": len(lat_ms)}


def run_server(server, reqs, rate_rps=None, seed=0xC4A, details=None):
    """Submit reqs at Poisson arrival times (all at once when rate is None)
    from one thread while another waits for completions. `details`, a
    list, receives per request (points, group, wave, arrival, submit, admit,
    done) in nanoseconds."""
    arr = poisson_arrivals(rate_rps, len(reqs), seed)
    tickets = [None] * len(reqs)
    arrival_ns = [0] * len(reqs)
    done = [None] * len(reqs)
    ready = queue.Queue()

    def waiter():
        for _ in range(len(reqs)):
            i = ready.get()
            done[i] = server.wait(tickets[i])

    th = threading.Thread(target=waiter)
    th.start()
    t0 = time.monotonic_ns()
    for i, r in enumerate(reqs):
        target = t0 + int(arr[i] * 1e9)
        while True:
            now = time.monotonic_ns()
            if now >= target:
                break
            time.sleep(min(0.002, (target - now) / 1e9))
        arrival_ns[i] = max(target, 0)
        tickets[i] = server.submit(r.group, r.n, r.G, r.out)
        ready.put(i)
    th.join()
    lat = [done[i]["done_ns"] - arrival_ns[i] for i in range(len(reqs))]
    if details is not None:
        for i, r in enumerate(reqs):
            d = done[i]
            details.append((r.n, r.k, d["wave"], arrival_ns[i], d["submit_ns"], d["admit_ns"], d["done_ns"]))
    pts = sum(r.n for r in reqs)
    return _summary(lat, pts, t0, max(d["done_ns"] for d in done))


def run_plain(torch, ss, reqs, rate_rps=None, seed=0xC4A):
    """The plain executor launched per request, one at a time in arrival
    order: pinned input copy, execute_batch, output copy, synchronize."""
    arr = poisson_arrivals(rate_rps, len(reqs), seed)
    stream = torch.cuda.Stream()
    # device buffers sized for the largest request, reused
    nmax = max(r.n for r in reqs)
    dP = torch.empty(3 * nmax, dtype=torch.float32, device="cuda")
    dout = torch.empty(4 * nmax, dtype=torch.float32, device="cuda")
    t0 = time.monotonic_ns()
    lat, last = [], t0
    for i, r in enumerate(reqs):
        target = t0 + int(arr[i] * 1e9)
        while time.monotonic_ns() < target:
            time.sleep(min(0.002, max(0.0, (target - time.monotonic_ns()) / 1e9)))
        with torch.cuda.stream(stream):
            p = dP[:3 * r.n].view(3, r.n)
            p.copy_(r.P, non_blocking=True)
            o = dout[:4 * r.n]
            o.zero_()
            G = make_globals(P=p)
            ss.execute_batch(r.group, r.n, G, 0, o.data_ptr(), stream.cuda_stream)
            r.out.copy_(o, non_blocking=True)
        stream.synchronize()
        last = time.monotonic_ns()
        lat.append(last - target)
    return _summary(lat, sum(r.n for r in reqs), t0, last)
