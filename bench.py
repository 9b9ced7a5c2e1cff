"""Benchmark: shading throughput of the GB300 executor.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

One step = one pass of the hot path (ShadingSystem batched execute of the
workload's shader group) over the workload's points, inputs resident in
HBM. Device time is measured with CUDA events on the launching stream
around each step; L2 is flushed (a 512 MiB write) between timed steps, so
every step reads its inputs from HBM. `e2e` repeats the measurement
through the public API with host buffers: pinned host->device copy of the
per-point inputs, the launch, device->host copy of the outputs.

--impl reference times the reference's batched CPU semantics on this
host's cores: the reference itself cannot be built here (LLVM, OIIO,
Imath absent) and its batched targets are x86-only, so the CPU port of
the reference algorithm (oracle/) stands in, with every host thread.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "Mpoints/s shaded at stated ulp match; p50/p99 latency: served vs plain GPU"
UNIT = "Mpoints/s"


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu, self.rows, self.proc = gpu, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


# ---- workloads ----------------------------------------------------------------------------
class FbmCell:
    """Single-layer pattern shader: 4-octave vector Perlin fBm with Dual2
    derivatives at P=(8u,8v,0) plus hash(cellnoise(P*4)); 1024x1024 grid,
    u,v at pixel centres; outputs Cout with x/y derivatives and the int."""
    name = "fbm_cell_1024x1024"
    rec = 10  # Cout val/dx/dy (9 floats) + cellhash

    def __init__(self, W=1024, H=1024):
        self.W, self.H, self.n = W, H, W * H
        self.name = "fbm_cell_%dx%d" % (W, H)

    def build(self, torch, og, shaders):
        from helpers import grid_globals, pixel_grid, single_layer_group
        self.ss = og.ShadingSystem()
        self.g = single_layer_group(self.ss, "fbm_cell", shaders.fbm_cell(), outputs=[
            og.SymLocationDesc("layer1.Cout", og.TypeColor, True, og.SymArenaOutputs, 0, 4 * self.rec),
            og.SymLocationDesc("layer1.cellhash", og.TypeInt, False, og.SymArenaOutputs, 36, 4 * self.rec)])
        self.ss.optimize_group(self.g)
        u, v = pixel_grid(self.W, self.H, centers=True)
        self.h_u, self.h_v = u, v
        self.d_uv = torch.from_numpy(np.stack([u, v])).cuda()
        self.G = grid_globals(self.d_uv[0], self.d_uv[1], self.W, self.H, centers=True)
        self.out = torch.zeros(self.n * self.rec, dtype=torch.float32, device="cuda")
        # e2e buffers: pinned host inputs and outputs
        self.pin_uv = torch.from_numpy(np.stack([u, v])).pin_memory()
        self.pin_out = torch.zeros(self.n * self.rec, dtype=torch.float32).pin_memory()
        self.G_host = grid_globals(self.pin_uv[0], self.pin_uv[1], self.W, self.H, centers=True)
        self.bytes_in = 8 * self.n
        self.bytes_out = 4 * self.rec * self.n

    def step(self, stream):
        self.ss.execute_batch(self.g, self.n, self.G, 0, self.out.data_ptr(), stream)

    def e2e_step(self, torch, stream):
        # host buffers in, host records out: the pipelined host-buffer entry
        self.ss.execute_batch_host(self.g, self.n, self.G_host, self.pin_out, 4 * self.rec)

    def algorithmic_bytes(self):
        # read u,v (8 B) + write Cout val/dx/dy (36 B) + cell hash (4 B)
        return 48 * self.n

    def lane_ops_per_point(self):
        # FP32+INT32 operations of the reference algorithm per point, counted
        # from its operation sequence: one Dual2<Vec3> 3-D Perlin lookup is
        # 1184 (floorfrac 9, 3 Dual2 fades 99, 8 lookup3 hashes 200, 3 channels
        # x (8 Dual2 grads 160 + Dual2 trilerp 128 + scale 3)), each octave adds
        # 45 for the Dual2 fBm accumulate; cell noise + hash + setup 80.
        return 4 * (1184 + 45) + 80

    def oracle_sample(self, oracle_run, og, n):
        from helpers import grid_globals
        n = min(n, self.n)
        G = grid_globals(self.h_u, self.h_v, self.W, self.H, centers=True)
        out = np.zeros((self.n, self.rec), np.float32)
        return lambda: oracle_run(self.g.program_bytes(), n, G, out)


class LayeredClosure:
    """3-layer connected group on 2048x2048 points: A simplex + cell noise on
    P*16, B an 8-knot catmull-rom color ramp driven by A, C the closure sum
    0.6*tint*diffuse(N) + 0.4*microfacet("ggx", N, dPdu, a, a, 1.5, 0); outputs
    the closure records and testrender's BSDF eval at normalize(1,1,1)."""
    name = "layered_closure_2048x2048"

    def __init__(self, W=2048, H=2048):
        from openshadinglanguage_gb300 import workloads
        self.wl = workloads
        self.W, self.H, self.n = W, H, W * H
        self.name = "layered_closure_%dx%d" % (W, H)
        self.rec = workloads.C2_STRIDE // 4

    def build_host(self, og, shaders):
        self.ss = og.ShadingSystem()
        self.g = self.wl.c2_group(self.ss)
        self.h_u, self.h_v, self.h_I = self.wl.c2_inputs(self.W, self.H)

    def build(self, torch, og, shaders):
        self.build_host(og, shaders)
        self.ss.optimize_group(self.g)
        self.d_in = torch.from_numpy(np.concatenate([self.h_u, self.h_v, self.h_I.ravel()])).cuda()
        n = self.n
        self.G = self.wl.c2_globals(og.make_globals, self.d_in[0:n], self.d_in[n:2 * n],
                                    self.d_in[2 * n:].view(3, n))
        self.out = torch.zeros(self.n * self.rec, dtype=torch.float32, device="cuda")
        self.pin_in = self.d_in.cpu().pin_memory()
        self.pin_out = torch.zeros(self.n * self.rec, dtype=torch.float32).pin_memory()
        self.G_host = self.wl.c2_globals(og.make_globals, self.pin_in[0:n], self.pin_in[n:2 * n],
                                         self.pin_in[2 * n:].view(3, n))
        self.bytes_in = 20 * self.n
        self.bytes_out = 4 * self.rec * self.n

    def step(self, stream):
        self.ss.execute_batch(self.g, self.n, self.G, 0, self.out.data_ptr(), stream)

    def e2e_step(self, torch, stream):
        # host buffers in, host records out: the pipelined host-buffer entry
        self.ss.execute_batch_host(self.g, self.n, self.G_host, self.pin_out, 4 * self.rec)

    def algorithmic_bytes(self):
        # read u, v, I (20 B) + write 2 closure records with count (132 B) + eval (16 B)
        return 168 * self.n

    def lane_ops_per_point(self):
        # 3-D simplex with one seed ~150, cell noise ~40, 8-knot catmull-rom
        # color spline ~70, closure construction and MULs ~60, BSDF walk +
        # prepare + diffuse and GGX eval with MIS ~230, layer glue ~30
        return 580

    def oracle_sample(self, oracle_run, og, n):
        n = min(n, self.n)
        G = self.wl.c2_globals(og.make_globals, self.h_u, self.h_v, self.h_I)
        out = np.zeros((self.n, self.rec), np.float32)
        return lambda: oracle_run(self.g.program_bytes(), n, G, out)


WORKLOADS = {FbmCell.name: FbmCell, LayeredClosure.name: LayeredClosure}
DEFAULT_WORKLOAD = LayeredClosure.name


def bench_batching(torch, og, reps=5, jit=1):
    """64 seeded random groups (20-200 ops, log-uniform 1K-1M points): the
    plain executor launched per group against the persistent batch launch
    (autotuned, CUDA-graph replay), interpreted and, with jit, as one
    persistent kernel specialized to the 64 programs. Same outputs bit for
    bit. The CPU figure is the oracle over a sample of every group's points
    on all host threads."""
    from openshadinglanguage_gb300 import workloads
    ss = og.ShadingSystem()
    specs = workloads.c3_specs()
    reqs = []
    for k, (name, oso, npts, _) in enumerate(specs):
        g = workloads.c3_group(ss, name, oso)
        dP = torch.from_numpy(workloads.c3_points(k, npts)).cuda()
        reqs.append((g, npts, og.make_globals(P=dP), dP, torch.zeros(npts * workloads.C3_REC, device="cuda")))
    total = sum(r[1] for r in reqs)
    st = torch.cuda.current_stream()
    sh = st.cuda_stream

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def plain():
        for g, n, G, _, o in reqs:
            ss.execute_batch(g, n, G, 0, o.data_ptr(), sh)

    t_plain = timed(plain)
    b = ss.batch()
    for g, n, G, _, o in reqs:
        b.add(g, n, G, 0, o.data_ptr())
    best, cands = b.autotune(sh, reps=2)
    b.set_launch(block=best["block"], heap_smem=best["heap_smem"], use_graph=True,
                 points_per_thread=best["points_per_thread"])
    t_batch = timed(lambda: b.execute(sh))
    b.close()
    ref = [o.cpu().numpy().copy() for (_, _, _, _, o) in reqs]
    out = {"workload": "64 random groups, %d points, seed 0xC3" % total, "points": total,
           "plain_ms": t_plain, "plain_mpts": total / t_plain / 1e3,
           "persistent_ms": t_batch, "persistent_mpts": total / t_batch / 1e3,
           "speedup_vs_plain": t_plain / t_batch,
           "autotuned": {k: best[k] for k in ("block", "points_per_thread", "heap_smem", "grid")},
           "candidates": len(cands), "launches_per_step": {"plain": len(reqs), "persistent": 1}}
    if jit:
        # the same requests with every group specialized (the reference's
        # per-group JIT): launched per group, and as one persistent kernel
        # specialized to the 64 programs
        ssj = og.ShadingSystem()
        ssj.attribute("jit", 1)
        gj = [workloads.c3_group(ssj, name, oso) for (name, oso, _, _) in specs]
        t0 = time.perf_counter()
        ssj.jit_groups(gj)
        t_groups = time.perf_counter() - t0
        jouts = [torch.zeros(npts * workloads.C3_REC, device="cuda") for (_, _, npts, _) in specs]

        def plain_jit():
            for k, g in enumerate(gj):
                ssj.execute_batch(g, specs[k][2], reqs[k][2], 0, jouts[k].data_ptr(), sh)

        t_plain_jit = timed(plain_jit)
        torch.cuda.synchronize()

        def same_as_plain():
            return all(bool(np.all((a == bb) | (np.isnan(a) & np.isnan(bb))))
                       for a, bb in zip(ref, (o.cpu().numpy() for o in jouts)))

        same_plain_jit = same_as_plain()
        for o in jouts:
            o.zero_()
        bj = ssj.batch()
        for k, g in enumerate(gj):
            bj.add(g, specs[k][2], reqs[k][2], 0, jouts[k].data_ptr())
        t0 = time.perf_counter()
        bestj, _ = bj.autotune(sh, reps=2)
        t_build = time.perf_counter() - t0
        bj.set_launch(block=bestj["block"], heap_smem=bestj["heap_smem"], use_graph=True, points_per_thread=1)
        t_jit = timed(lambda: bj.execute(sh))
        torch.cuda.synchronize()
        same = same_as_plain()
        bj.close()
        out.update({"plain_jit_ms": t_plain_jit, "plain_jit_mpts": total / t_plain_jit / 1e3,
                    "persistent_jit_ms": t_jit, "persistent_jit_mpts": total / t_jit / 1e3,
                    "jit_speedup_vs_plain": t_plain / t_jit,
                    "persistent_jit_over_plain_jit": t_plain_jit / t_jit,
                    "jit_groups_build_s": t_groups, "jit_batch_build_and_tune_s": t_build,
                    "jit_block": bestj["block"], "jit_same_bits_as_plain": same and same_plain_jit})
    out["cpu"] = c3_cpu_baseline(og, workloads, specs)
    return out


def c3_cpu_baseline(og, workloads, specs, frac=2, min_s=2.0):
    """The oracle over every group's first n/frac points (at least 2000) on
    all host threads, repeated until at least min_s seconds of work: points
    per second over the sampled points."""
    from helpers import oracle_run
    from oracle.build import build as build_oracle
    build_oracle()
    ss = og.ShadingSystem()
    work = []
    for k, (name, oso, npts, _) in enumerate(specs):
        g = workloads.c3_group(ss, name, oso)
        m = min(npts, max(2000, npts // frac))
        P = np.ascontiguousarray(workloads.c3_points(k, npts)[:, :m])
        work.append((g.program_bytes(), m, og.make_globals(P=P), P, np.zeros((m, workloads.C3_REC), np.float32)))
    pts, secs, rounds = 0, 0.0, 0
    while secs < min_s:
        for blob, m, G, _, buf in work:
            t0 = time.perf_counter()
            oracle_run(blob, m, G, buf)
            secs += time.perf_counter() - t0
            pts += m
        rounds += 1
    return {"mpts_per_s": pts / secs / 1e6, "points": pts, "seconds": secs, "threads": os.cpu_count(),
            "kind": "port", "sample": "first n/%d points (at least 2000) of each of the 64 groups, %d rounds"
            % (frac, rounds)}


def bench_serving(torch, og, nreq=600, jit=0):
    """Poisson request stream over the 64 groups (point counts log-uniform
    in [256, 262144]) at 10/50/90/100% of the server's measured peak, served
    with continuous batching and by the plain executor per request."""
    from openshadinglanguage_gb300 import serving, workloads
    ss = og.ShadingSystem()
    groups = [workloads.c3_group(ss, name, oso) for (name, oso, _, _) in workloads.c3_specs()]
    reqs = serving.make_requests(torch, groups, nreq)
    srv = ss.server(budget_bytes=40 << 30, streams=3)
    for g in groups:
        srv.register(g)
    serving.run_server(srv, reqs[:50])
    peak = serving.run_server(srv, reqs)
    peak_rps = len(reqs) / peak["makespan_s"]
    plain_peak = serving.run_plain(torch, ss, reqs)
    loads = {}
    for frac in (0.1, 0.5, 0.9, 1.0):
        rate = frac * peak_rps
        a = serving.run_server(srv, reqs, rate_rps=rate)
        p = serving.run_plain(torch, ss, reqs, rate_rps=rate)
        loads["%d%%" % int(frac * 100)] = {
            "offered_rps": rate,
            "served": {k: a[k] for k in ("p50_ms", "p99_ms", "throughput_mpts")},
            "plain": {k: p[k] for k in ("p50_ms", "p99_ms", "throughput_mpts")}}
    st = srv.stats()
    srv.close()
    out = {"requests": nreq, "points": sum(r.n for r in reqs), "hbm_budget_gb": 40,
           "peak_rps": peak_rps, "served_peak_mpts": peak["throughput_mpts"],
           "plain_peak_mpts": plain_peak["throughput_mpts"], "loads": loads,
           "arena_high_water_mb": st["arena_high_water"] / 2 ** 20, "waves": st["waves"],
           "latency": "arrival to outputs in host memory (pinned), host monotonic clock"}
    if jit:
        # waves on one kernel specialized to the 64 programs (the same
        # programs as the batching section: its cached kernel)
        ssj = og.ShadingSystem()
        ssj.attribute("jit", 1)
        gj = [workloads.c3_group(ssj, name, oso) for (name, oso, _, _) in workloads.c3_specs()]
        jreqs = serving.make_requests(torch, gj, nreq)
        srvj = ssj.server(budget_bytes=40 << 30, streams=3)
        for g in gj:
            srvj.register(g)
        t0 = time.perf_counter()
        serving.run_server(srvj, jreqs[:50])
        t_build = time.perf_counter() - t0
        pj = serving.run_server(srvj, jreqs)
        aj = serving.run_server(srvj, jreqs, rate_rps=0.9 * peak_rps)
        srvj.close()
        out.update({"served_jit_peak_mpts": pj["throughput_mpts"],
                    "served_jit_over_plain_peak": pj["throughput_mpts"] / plain_peak["throughput_mpts"],
                    "served_jit_at_90pct": {k: aj[k] for k in ("p50_ms", "p99_ms", "throughput_mpts")},
                    "served_jit_first_wave_s": t_build})
    return out


def host_link_peak(torch, bytes_in, bytes_out, reps=5):
    """The host link's copy peaks for the e2e step's byte counts: plain
    cudaMemcpyAsync of pinned host buffers of bytes_in (H2D) and bytes_out
    (D2H), each alone, then both at once on two streams; the floor of the
    e2e step is its copies at these rates."""
    h_in = torch.empty(bytes_in // 4, dtype=torch.float32).pin_memory()
    h_out = torch.empty(bytes_out // 4, dtype=torch.float32).pin_memory()
    d_in = torch.empty_like(h_in, device="cuda")
    d_out = torch.empty_like(h_out, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return min(ts)

    def both():
        with torch.cuda.stream(s1):
            d_in.copy_(h_in, non_blocking=True)
        with torch.cuda.stream(s2):
            h_out.copy_(d_out, non_blocking=True)
    t_h2d = timed(lambda: d_in.copy_(h_in, non_blocking=True))
    t_d2h = timed(lambda: h_out.copy_(d_out, non_blocking=True))
    t_both = timed(both)
    return {"h2d_gbs": bytes_in / t_h2d / 1e9, "d2h_gbs": bytes_out / t_d2h / 1e9,
            "duplex_ms": 1e3 * t_both, "ms_floor": 1e3 * t_both,
            "method": "pinned cudaMemcpyAsync, best of %d, host clock" % reps}


def bench_wavefront(torch, og, frames=3, cpu_step=97, size=None, jit=1):
    """Wavefront path tracing of the seeded 1000-primitive scene with the 16
    layered materials: 1920x1080x4 paths, up to 8 hits, Russian roulette
    survival 0.8. A frame (all bounces) is one CUDA-graph replay; a
    profiled frame gives the per-stage split. The oracle's path loop renders
    every cpu_step-th path on all host threads for the CPU figure."""
    from openshadinglanguage_gb300 import workloads
    from helpers import oracle_wavefront
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)  # materials shade in a batch kernel specialized to them (built at create)
    mats = workloads.c5_materials(ss)
    prims = workloads.c5_scene()
    dims = {}
    if size:
        w, h, spp = (int(x) for x in size.split("x"))
        dims = dict(width=w, height=h, spp=spp)
    t_build = time.perf_counter()
    wf = ss.wavefront(prims, mats, **dims)
    t_build = time.perf_counter() - t_build
    o = wf.options
    rad = torch.empty(3 * wf.paths, dtype=torch.float32, device="cuda")
    img = torch.empty(o["width"] * o["height"] * 3, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream()
    for _ in range(2):
        wf.render(rad.data_ptr(), img.data_ptr(), st.cuda_stream)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(frames)]
    for a, b in evs:
        a.record(st)
        wf.render(rad.data_ptr(), img.data_ptr(), st.cuda_stream)
        b.record(st)
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
    s = wf.stats()
    wf.render(rad.data_ptr(), img.data_ptr(), st.cuda_stream, profile=True)
    prof = wf.stats()
    status = ss.device_status()
    nhits = s["total_hits"]
    # CPU: the oracle's path loop over a strided sample of the same frame,
    # the stride shrunk until the sample takes at least 2 s
    oracle_wavefront(o, prims, mats, begin=0, step=cpu_step * 8)  # warm-up on a smaller sample
    while True:
        t0 = time.perf_counter()
        crad, chits, _ = oracle_wavefront(o, prims, mats, begin=0, step=cpu_step)
        cpu_s = time.perf_counter() - t0
        if cpu_s >= 2.0 or cpu_step == 1:
            break
        cpu_step = max(1, int(cpu_step * cpu_s / 3.0))
    ncpu = crad.shape[1]
    wf.close()
    stages = dict(zip(("trace", "plan", "scatter", "shade", "update"), prof["ms_stage"]))
    return {"workload": "wavefront %dx%dx%d spp, <=8 hits, RR 0.8, 1000 spheres/rectangles seed 0xC5, "
                        "16 materials" % (o["width"], o["height"], o["spp"]), "paths": wf.paths, "frame_ms": ms,
            "mpaths_per_s": wf.paths / ms / 1e3, "shading_points": nhits,
            "mhits_per_s": nhits / ms / 1e3, "hits_per_bounce": s["hits"][:o["max_hits"]],
            "profiled_stage_ms": stages, "device_status": status,
            "shading_kernel": "specialized batch kernel (jit)" if jit else "interpreter batch kernel",
            "create_s": t_build,
            "launches_per_frame": 2 + 5 * o["max_hits"] + 1,
            "cpu": {"paths": ncpu, "hits": int(chits.sum()), "seconds": cpu_s,
                    "mpaths_per_s": ncpu / cpu_s / 1e6, "mhits_per_s": float(chits.sum()) / cpu_s / 1e6,
                    "threads": os.cpu_count(), "kind": "port",
                    "sample": "every %dth path of the frame, oracle path loop (brute-force intersection, "
                              "batched shading per material)" % cpu_step}}


def bench_texture(torch, og, reps=10):
    """texture() throughput: a 2048x2048 grid looking up a registered
    1024x1024 RGB image (4 MB level 0, 11-level pyramid) at s, t = 1.7 u,
    1.7 v (footprint between levels 0 and 1: two bilinear lookups blended),
    periodic wrap; interpreter and specialized kernel; the oracle on a
    sample of the points on all host threads. Image and grid stay in L2
    between launches (4 MB + 32 MB in, 50 MB out): the number is the
    filter's arithmetic rate, not an HBM figure."""
    from helpers import grid_globals, oracle, oracle_run, pixel_grid, single_layer_group
    from openshadinglanguage_gb300.shaders import texture_lookup as tex_shader
    import ctypes
    img = np.random.default_rng(7).random((1024, 1024, 3), dtype=np.float32)
    W = H = 2048
    n = W * H
    u, v = pixel_grid(W, H, centers=True)
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    out = torch.empty(n * 3, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream()
    res = {"workload": "texture 2048x2048 lookups of a 1024x1024 RGB float image, trilinear, periodic"}
    for jit in (0, 1):
        ss = og.ShadingSystem()
        if jit:
            ss.attribute("jit", 1)
        idx = ss.texture_create("img", img)
        g = single_layer_group(ss, "btex", tex_shader("btex", 1.7, "periodic"),
                               outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
        G = grid_globals(du, dv, W, H, centers=True)
        for _ in range(3):
            ss.execute_batch(g, n, G, 0, out.data_ptr(), st.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            ss.execute_batch(g, n, G, 0, out.data_ptr(), st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        res["specialized" if jit else "interpreter"] = {"ms": ms, "mpts_per_s": n / ms / 1e3,
                                                         "device_status": ss.device_status()}
        if not jit:
            L = oracle()
            L.oracle_texture_create.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p]
            L.oracle_texture_create(idx, 1024, 1024, 3, img.ctypes.data)
            m = 1 << 20
            ref = np.zeros((m, 3), np.float32)
            Gh = grid_globals(u[:m], v[:m], W, H, centers=True)
            t0 = time.perf_counter()
            oracle_run(g.program_bytes(), m, Gh, ref)
            dt = time.perf_counter() - t0
            res["cpu"] = {"mpts_per_s": m / dt / 1e6, "points": m, "threads": os.cpu_count(), "kind": "port"}
        out.zero_()
        ss.execute_batch(g, n, G, 0, out.data_ptr(), st.cuda_stream)
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(n, 3)[:m]
        res["specialized" if jit else "interpreter"]["bit_exact_sample"] = bool(
            np.array_equal(got.view(np.uint32), ref.view(np.uint32)))
    return res


def cpu_reference(wl, og, budget_s=2.0):
    """Time the CPU port of the reference semantics on all host threads."""
    from helpers import oracle_run
    n = 4096
    while True:
        run = wl.oracle_sample(oracle_run, og, n)
        t0 = time.perf_counter()
        run()
        dt = time.perf_counter() - t0
        if dt > 0.25 * budget_s or n >= wl.n:
            break
        n = min(wl.n, n * 4)
    reps = max(1, int(budget_s / max(dt, 1e-6)))
    t0 = time.perf_counter()
    for _ in range(reps):
        run()
    dt = (time.perf_counter() - t0) / reps
    return n / dt / 1e6, n, reps


def progress(msg):
    """A timestamped progress line on stderr (the JSON line is stdout's only line)."""
    print("[bench %s] %s" % (time.strftime("%H:%M:%S"), msg), file=sys.stderr, flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--size", type=int, default=0,
                    help="grid width = height override (a smaller case of the workload, e.g. for profiling)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the 64-group batching, serving and wavefront measurements")
    ap.add_argument("--jit", type=int, default=1,
                    help="1: run the group's specialized kernel (attribute jit), 0: the interpreter")
    ap.add_argument("--jit-block", type=int, default=0, help="specialized launch: threads per CTA")
    ap.add_argument("--jit-pool-smem", type=int, default=-1, help="specialized launch: closure pools in smem (1/0)")
    ap.add_argument("--host-direct", type=int, default=1,
                    help="e2e: the kernel writes pinned host output records directly (1) or via copies (0)")
    ap.add_argument("--jit-min-blocks", type=int, default=0,
                    help="specialized kernel register cap: 256-thread CTAs per SM it must fit (2..8)")
    ap.add_argument("--section", choices=["batching", "serving", "wavefront", "texture"],
                    help="run only this measurement section and print it as one JSON line")
    ap.add_argument("--wf-size", default=None, help="wavefront frame WxHxSPP (default 1920x1080x4)")
    ap.add_argument("--batch-jit", type=int, default=1,
                    help="batching and serving sections: also time every group specialized (per group, "
                         "one persistent kernel for the 64 programs, and served waves on that kernel); "
                         "about 100 s of kernel builds on a cold cache")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.section:
        import torch
        import openshadinglanguage_gb300 as og
        from openshadinglanguage_gb300.build import build as build_native
        build_native()
        torch.cuda.set_device(0)
        fn = {"batching": lambda: bench_batching(torch, og, jit=args.batch_jit),
              "serving": lambda: bench_serving(torch, og, jit=args.batch_jit),
              "wavefront": lambda: bench_wavefront(torch, og, size=args.wf_size, jit=args.jit),
              "texture": lambda: bench_texture(torch, og)}[args.section]
        print(json.dumps({"section": args.section, args.section: fn()}))
        return 0

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    import openshadinglanguage_gb300 as og
    from openshadinglanguage_gb300 import shaders
    from oracle.build import build as build_oracle

    wl = WORKLOADS[args.workload](args.size, args.size) if args.size > 0 else WORKLOADS[args.workload]()

    if args.impl == "reference":
        if rank != 0:
            return 0
        build_oracle()
        import torch  # noqa: F401  (import order matches the GPU arm)
        # the oracle needs the lowered program; lowering is host-only
        wl.ss = og.ShadingSystem()
        from helpers import single_layer_group  # noqa: F401
        wl.build_host_only = True
        _build_host(wl, og, shaders)
        rates = []
        for _ in range(args.warmup):
            cpu_reference(wl, og, budget_s=0.5)
        for _ in range(args.steps):
            r, n, reps = cpu_reference(wl, og, budget_s=1.0)
            rates.append(r)
        v = float(np.mean(rates))
        cores = os.cpu_count()
        line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * n / (v * 1e6), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": wl.name, "points": wl.n, "sample_points_per_step": n},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": "%d of %d points per step, OpenMP over %d threads" % (n, wl.n, cores)},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "reference batched CPU path not buildable here (LLVM/OIIO/Imath absent) and x86-only; "
                        "timed: the CPU port of its semantics (oracle/)"}
        print(json.dumps(line))
        return 0

    import torch
    from openshadinglanguage_gb300.build import build as build_native
    build_native()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    progress("building %s" % wl.name)
    wl.build(torch, og, shaders)
    if args.jit:
        wl.ss.attribute("jit", 1)  # the first launch (warm-up) builds and loads the kernel
        if args.jit_block:
            wl.ss.attribute("jit_block", args.jit_block)
        if args.jit_pool_smem >= 0:
            wl.ss.attribute("jit_pool_smem", args.jit_pool_smem)
        if args.jit_min_blocks:
            wl.ss.attribute("jit_min_blocks", args.jit_min_blocks)
        wl.ss.attribute("host_direct_outputs", args.host_direct)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    for _ in range(args.warmup):
        wl.step(sh)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    with ClockSampler(local_rank) as clk:
        # nvidia-smi needs a moment to start sampling; keep the GPU busy meanwhile
        t_start = time.time()
        while time.time() - t_start < 0.6:
            wl.step(sh)
            torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()
            evs[i][0].record(stream)
            wl.step(sh)
            evs[i][1].record(stream)
        barrier()
    times = [a.elapsed_time(b) for a, b in evs]  # ms
    total_ms = float(np.sum(times))
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = wl.n * world / (ms_per_step * 1e-3) / 1e6
    status = wl.ss.device_status()

    # end to end through the public API with host buffers
    progress("e2e")
    for _ in range(2):
        wl.e2e_step(torch, sh)
    torch.cuda.synchronize()
    # the host-buffer call returns when the outputs are in host memory: timed
    # on the host clock, device idle and L2 flushed before each call
    e_times = []
    barrier()
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        wl.e2e_step(torch, sh)
        e_times.append(time.perf_counter() - t0)
    barrier()
    e_ms = 1e3 * float(np.mean(e_times))
    e2e_value = wl.n * world / (e_ms * 1e-3) / 1e6
    link = host_link_peak(torch, wl.bytes_in, wl.bytes_out)

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    peaks = _peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    clocks = clk.summary()
    achieved_gbs = wl.algorithmic_bytes() / (ms_per_step * 1e-3) / 1e9
    ops = wl.lane_ops_per_point() * wl.n / (ms_per_step * 1e-3) / 1e12
    mhz_max = peaks.get("sm_max_mhz", 2070.0)
    mhz_load = clocks.get("sm_mhz") or peaks.get("clocks_under_load", {}).get("sm_mhz_median", 1417.0)
    alu_peak_max = sms * 128 * mhz_max * 1e6 / 1e12
    alu_peak_load = sms * 128 * mhz_load * 1e6 / 1e12
    traffic = None
    prof = os.path.join(ROOT, "profiles", "traffic_%s.json" % wl.name)
    if os.path.exists(prof):
        traffic = json.load(open(prof)).get("bytes_per_launch")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl.name, "points": wl.n, "l2": "flushed (512 MiB write) between timed steps",
                   "kernel": "specialized per group (jit)" if args.jit else "interpreter",
                   "parity": "bit-exact to the CPU oracle (non-FMA reference order) for floats and ints"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": wl.bytes_in,
                "d2h_bytes_per_step": wl.bytes_out, "ms_per_step": e_ms,
                "link": dict(link, frac=link["ms_floor"] / e_ms,
                             note="frac = the step's copies at the measured link peaks (H2D and D2H "
                                  "overlapped) / the e2e step")},
        "gpu_launches": args.steps,
        "clocks": clocks,
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s",
                     "frac": achieved_gbs / hbm, "traffic": traffic,
                     "note": "of measured HBM peak; the interpreter is ALU-issue bound, see roofline_alu"},
        "roofline_alu": {"bound": "alu", "achieved": ops, "unit": "Tlane-op/s",
                         "ops_per_point": wl.lane_ops_per_point(),
                         "peak_at_max_clock": alu_peak_max, "frac_at_max_clock": ops / alu_peak_max,
                         "peak_at_sampled_clock": alu_peak_load, "frac_at_sampled_clock": ops / alu_peak_load,
                         "sms": sms},
        "device_status": status,
    }
    if not args.no_extras and world == 1:
        progress("batching")
        line["batching"] = bench_batching(torch, og, jit=args.batch_jit)
        progress("serving")
        line["serving"] = bench_serving(torch, og, jit=args.batch_jit)
        progress("wavefront")
        line["wavefront"] = bench_wavefront(torch, og, jit=args.jit)
        progress("texture")
        line["texture"] = bench_texture(torch, og)
        progress("sections done")
        # the systems targets as top-level keys, ahead of the long sections
        b, sv = line["batching"], line["serving"]
        summary = {"speedup_vs_plain": b["speedup_vs_plain"],
                   "jit_speedup_vs_plain": b.get("jit_speedup_vs_plain"),
                   "persistent_jit_over_plain_jit": b.get("persistent_jit_over_plain_jit"),
                   "served_over_plain_peak": sv["served_peak_mpts"] / sv["plain_peak_mpts"],
                   "served_jit_over_plain_peak": sv.get("served_jit_over_plain_peak")}
        keys = list(line)
        at = keys.index("ms_per_step") + 1
        line = dict([(k, line[k]) for k in keys[:at]] + list(summary.items()) + [(k, line[k]) for k in keys[at:]])
    if not args.no_cpu_baseline:
        from helpers import oracle_run  # noqa: F401
        build_oracle()
        r, n, reps = cpu_reference(wl, og, budget_s=2.0)
        line["cpu_baseline"] = {"value": r, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "sample": "%d of %d points, %d reps, OpenMP over all host threads" % (n, wl.n, reps)}
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def _build_host(wl, og, shaders):
    """Host-only setup for the CPU arm: lower the group and make inputs."""
    from helpers import pixel_grid, single_layer_group
    if hasattr(wl, "build_host"):
        wl.build_host(og, shaders)
        return
    if isinstance(wl, FbmCell):
        wl.g = single_layer_group(wl.ss, "fbm_cell", shaders.fbm_cell(), outputs=[
            og.SymLocationDesc("layer1.Cout", og.TypeColor, True, og.SymArenaOutputs, 0, 4 * wl.rec),
            og.SymLocationDesc("layer1.cellhash", og.TypeInt, False, og.SymArenaOutputs, 36, 4 * wl.rec)])
        wl.h_u, wl.h_v = pixel_grid(wl.W, wl.H, centers=True)


if __name__ == "__main__":
    sys.exit(main())
