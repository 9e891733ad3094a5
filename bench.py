"""Benchmark of the photon-propagation path on the 60x60x30 mm inclusion phantom
(648 000 tetrahedra, 1 mm grid, Gaussian sigma = 1 mm direct source, Fresnel boundary).

A step is one simulation of ``--photons`` photons (default 1e8) through the FP32 tracking
form with the mesh resident on the device.  Reported:
  value       photons/s with the mesh and job resident (whole-job: setup of the job,
              kernel, read-back), max over ranks
  e2e         photons/s through vmc_run with host buffers: setup, uploads, kernel and the
              read-back of all results inside the timed region
  fp64        the plain FP64 form on the same workload (photons/s) and the ratio
  roofline    the pool kernel's algorithmic gather bytes (108 B per CW element step, the
              per-step record of the reference layout) over its CUDA-event duration,
              against the measured HBM copy bandwidth; the measured L2 random-gather
              ceiling is reported beside it
  cpu_baseline the CPU oracle (OpenMP restatement of the reference engine) on all host
              cores on a bounded sample of the same workload
  matched_error  chi2/dof of FP32-form batch means against FP64-form batch means (1 means
              the FP32 form has no error beyond the Monte Carlo noise)
  serve       p50/p99 latency and photons/s of a short Poisson request stream
The L2 (129 MB) is flushed between timed steps by writing a 512 MB buffer.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_STEP_CW = 108  # element nodes 16 + coordinates 48 + HN row 16 + optics 12 + ER RMW 16
METRIC = "photons/s FP32-track vs FP64 GPU at matched fluence error; serve p50/p99 latency"
WORKLOAD = "inclusion phantom 60x60x30 mm, 648000 tets, gaussian sigma 1 mm direct source, CW"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max over ranks (torch.distributed); trivial with one rank."""

    def __init__(self, ws):
        self.ws = ws
        if ws > 1:
            import torch.distributed as td
            backend = "nccl" if os.environ.get("VMC_DIST_BACKEND", "gloo") == "nccl" else "gloo"
            td.init_process_group(backend=backend)
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, v):
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def flush_l2():
    """Write a 512 MB device buffer (4x the L2) between timed steps."""
    import torch
    if not hasattr(flush_l2, "buf"):
        flush_l2.buf = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    flush_l2.buf.fill_(1)
    torch.cuda.synchronize()


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fp:
            d = json.load(fp)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per element step of the FP32 pool kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "pool_kernel_fp32_phantom.json")
    if os.path.exists(path):
        with open(path) as fp:
            d = json.load(fp)
        return d.get("dram_bytes_per_step")
    return None


def cpu_baseline(p, seconds_target=12.0, threads=None, name="phantom"):
    """The CPU oracle on all host cores, on a sample sized to ~seconds_target of work."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    threads = threads or os.cpu_count() or 1
    probe = max(threads * 400, 2000)
    r = oracle.run(p, rng=oracle.RNG_MT, nthreads=threads, nphoton=probe, normalize=False)
    rate = probe / max(r.seconds, 1e-6)
    n = int(min(max(rate * seconds_target, probe), 5e6))
    r = oracle.run(p, rng=oracle.RNG_MT, nthreads=threads, nphoton=n, normalize=False)
    rate = n / r.seconds
    return {"value": rate, "unit": "photons/s", "cores": threads, "kind": "port",
            "sample": f"{n} photons of the {name} workload (MT19937, {threads} OpenMP threads), "
                      f"{r.seconds:.1f} s", "steps_per_photon": r.steps / n}


def reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from valomc_gb300 import meshgen as mg
    p = mg.config_3d_phantom(nphoton=1, seed=12345)
    vals = []
    base = None
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(p, seconds_target=args.ref_seconds)
        if i >= args.warmup:
            vals.append(b["value"])
            base = b
    v = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "photons/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * args.ref_seconds,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD},
            "cpu_baseline": {"value": v, "unit": "photons/s", "cores": base["cores"], "kind": "port",
                             "sample": base["sample"]},
            "e2e": {"value": v, "unit": "photons/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def serve_run(seconds, rate_hz, seed=5):
    """Poisson request stream against resident meshes (smaller budgets than the full mix so
    the run stays short): returns latency percentiles and aggregate photons/s."""
    import valomc_gb300 as V
    from valomc_gb300 import meshgen as mg
    rng = np.random.default_rng(seed)
    sizes = [12, 16, 20, 24]
    meshes, probs = [], []
    for L in sizes:
        p = mg.pencil_box(L, 0.02, 10.0, 0.9, 1.4, (L / 2 + 0.3, L / 2 + 0.2), 1, seed=1)
        meshes.append(V.Mesh(p))
        probs.append(p)
    srv = V.Server(max_slots=64, memory_budget=4 << 30)
    ids = [srv.add_mesh(m) for m in meshes]
    t0 = time.time()
    sub = []
    t = 0.0
    while t < seconds:
        t += rng.exponential(1.0 / rate_hz)
        k = int(rng.integers(len(sizes)))
        p = probs[k].copy()
        p.mua[:] = rng.uniform(0.005, 0.1)
        p.mus[:] = rng.uniform(5, 20)
        p.g[:] = rng.uniform(0.8, 0.95)
        p.n[:] = rng.uniform(1.33, 1.45)
        nph = int(math.exp(rng.uniform(math.log(1e4), math.log(1e6))))
        now = time.time() - t0
        if t > now:
            time.sleep(t - now)
        sub.append((srv.submit(ids[k], p, nphoton=nph, seed=int(rng.integers(1 << 30))), nph, time.time()))
    lat, tot = [], 0
    for rid, nph, ts in sub:
        r = srv.wait(rid)
        lat.append(r.stats["seconds_total"])
        tot += nph
    wall = time.time() - t0
    srv.close()
    return {"requests": len(sub), "rate_hz": rate_hz, "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "photons_per_s": tot / wall,
            "note": "Poisson arrivals; cubes 12-24 mm, photons log-uniform 1e4-1e6, config-4 optics"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--photons", type=float, default=1e8)
    ap.add_argument("--fp64-photons", type=float, default=1e7)
    ap.add_argument("--ref-seconds", type=float, default=10.0)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--serve-seconds", type=float, default=6.0)
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--config", default="phantom", choices=["phantom", "fd", "batch", "serve", "square2d"],
                    help="phantom: the headline line; fd / batch / serve: the other workloads, one line each")
    ap.add_argument("--batch-photon-scale", type=float, default=1.0)
    ap.add_argument("--serve-rate", type=float, default=50.0)
    ap.add_argument("--serve-window", type=float, default=10.0)
    ap.add_argument("--serve-epoch", type=float, default=0.0,
                    help="photons per serving epoch (0: the loop's own choice, 50 ms to 0.5 s of work by backlog)")
    ap.add_argument("--serve-slots", type=int, default=64, help="requests the serving loop simulates at once")
    ap.add_argument("--serve-block", type=int, default=0, help="threads per CTA of the serving launches (0: default)")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.config != "phantom":
        return {"fd": bench_fd, "batch": bench_batch, "serve": bench_serve, "square2d": bench_square2d}[args.config](args)

    ws, rank, local = dist_env()
    dist = Dist(ws)
    import valomc_gb300 as V
    from valomc_gb300 import meshgen as mg
    dev = local
    nph = int(args.photons)
    p = mg.config_3d_phantom(nphoton=nph, seed=12345)
    # replicas: disjoint photon index ranges of one Philox stream per rank
    offset = rank * nph
    mesh = V.Mesh(p, precision=V.VMC_FP32, device=dev)
    opts = V.options(precision=V.VMC_FP32, device=dev, photon_offset=offset)

    def step():
        res, tot = V.run_batch([mesh], [p], opts=opts)
        return res[0], tot

    for _ in range(args.warmup):
        step()
        flush_l2()
    kernel_s, steps_tot, wall = [], 0, 0.0
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush_l2()
            dist.barrier()
            t0 = time.perf_counter()
            r, tot = step()
            t1 = time.perf_counter()
            dist.barrier()
            wall += t1 - t0
            kernel_s.append(tot["seconds_kernel"])
            steps_tot += tot["steps"]
    wall_max = dist.max(wall)
    photons_all = dist.sum(nph * args.steps)
    value = photons_all / wall_max
    kmean = float(np.mean(kernel_s))
    steps_per_launch = steps_tot / args.steps

    # e2e: the reference-facing call with host buffers (setup + H2D + kernel + D2H inside)
    e2e_wall = 0.0
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        flush_l2()
        dist.barrier()
        t0 = time.perf_counter()
        re = V.run(p, precision=V.VMC_FP32, device=dev, photon_offset=offset)
        e2e_wall += time.perf_counter() - t0
    e2e_value = dist.sum(nph * e2e_steps) / dist.max(e2e_wall)
    h2d = re.stats["bytes_h2d"]
    d2h = re.stats["bytes_d2h"]

    out = None
    if rank == 0:
        peak, peak_kind = measured_peaks()
        achieved = BYTES_PER_STEP_CW * steps_per_launch / kmean / 1e9
        traffic_per_step = ncu_traffic()
        line = {
            "metric": METRIC, "value": value, "unit": "photons/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * wall_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "photons_per_step": nph, "precision": "fp32-track",
                       "accumulation": "f64",
                       "l2": "flushed between steps (512 MB write)", "replicas": ws},
            "tet_steps_per_s": steps_per_launch / kmean,
            "steps_per_photon": steps_per_launch / nph,
            "kernel_s_per_step": kmean,
            "gpu_launches": args.steps,
            "e2e": {"value": e2e_value, "unit": "photons/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind,
                         "traffic": (traffic_per_step * steps_per_launch) if traffic_per_step else None,
                         "algorithmic_bytes_per_launch": BYTES_PER_STEP_CW * steps_per_launch},
            "clocks": clk.summary(),
        }
        if not args.no_extras:
            gather = V.bench_gather(int(p.Ne * 80 + p.Ne * 16), seconds=0.3, device=dev)
            line["roofline"]["l2_gather_peak_gbs"] = gather
            line["roofline"]["l2_gather_frac"] = achieved / gather
            # plain FP64 form on the same mesh
            n64 = int(args.fp64_photons)
            V.run(p, precision=V.VMC_FP64, device=dev, nphoton=min(n64, 1_000_000))  # warm-up
            r64b = V.run(p, precision=V.VMC_FP64, device=dev, nphoton=n64, seed=777)
            fp64_rate = n64 / r64b.stats["seconds_kernel"]
            fp32_rate = nph / kmean
            line["fp64"] = {"photons_per_s": fp64_rate, "tet_steps_per_s": r64b.stats["steps"] / r64b.stats["seconds_kernel"],
                            "fp32_over_fp64": fp32_rate / fp64_rate, "fp64_tflops_peak": V.bench_fp64(0.2, dev)}
            line["matched_error"] = matched_error(V, p, dev)
            line["cpu_baseline"] = cpu_baseline(p, seconds_target=args.cpu_seconds)
            line["cpu_baseline"]["gpu_over_cpu"] = value / line["cpu_baseline"]["value"]
            if args.serve_seconds > 0:
                line["serve"] = serve_run(args.serve_seconds, 50.0)
        out = line
        print(json.dumps(out), flush=True)
    dist.close()
    return 0


def bench_fd(args):
    """The frequency-domain phantom (per-tet lognormal mua, U(8, 12) mus, 100 MHz): both forms."""
    import valomc_gb300 as V
    from valomc_gb300 import meshgen as mg
    p = mg.config_3d_fd(nphoton=int(args.photons), seed=12345)
    out = {"metric": "photons/s, frequency-domain phantom", "unit": "photons/s",
           "config": {"workload": "FD phantom 648000 tets, f = 100 MHz, lognormal mua, U(8,12) mus"}}
    for prec, name, n in ((V.VMC_FP32, "fp32", int(args.photons)), (V.VMC_FP64, "fp64", int(args.fp64_photons))):
        mesh = V.Mesh(p, precision=prec)
        q = p.copy(Nphoton=n)
        V.run_batch([mesh], [q], precision=prec)
        ks, st = [], None
        for _ in range(max(1, args.steps)):
            flush_l2()
            _, st = V.run_batch([mesh], [q], precision=prec)
            ks.append(st["seconds_kernel"])
        k = float(np.median(ks))
        out[name] = {"photons_per_s": n / k, "tet_steps_per_s": st["steps"] / k, "steps_per_photon": st["steps"] / n,
                     "achieved_gbs_128B_per_step": 128 * st["steps"] / k / 1e9}
        mesh.close()
    out["value"] = out["fp32"]["photons_per_s"]
    out["fp32_over_fp64"] = out["fp32"]["photons_per_s"] / out["fp64"]["photons_per_s"]
    print(json.dumps(out), flush=True)
    return 0


def bench_square2d(args):
    """The 2D square (10x10 mm, 200 triangles, cosinic source on edges 4..7, 1e6 photons):
    both forms through vmc_run (host buffers), and the CPU oracle on all host cores."""
    import valomc_gb300 as V
    from valomc_gb300 import meshgen as mg
    p = mg.config_2d_square(nphoton=1_000_000, seed=12345)
    out = {"metric": "photons/s, 2D square", "unit": "photons/s",
           "config": {"workload": "10x10 mm square, 200 triangles, cosinic edges 4-7, 1e6 photons"}}
    for prec, name in ((V.VMC_FP64, "fp64"), (V.VMC_FP32, "fp32")):
        V.run(p, precision=prec)
        rs = [V.run(p, precision=prec) for _ in range(max(1, args.steps))]
        k = min(r.stats["seconds_kernel"] for r in rs)
        tot = min(r.stats["seconds_total"] for r in rs)
        out[name] = {"photons_per_s_kernel": p.Nphoton / k, "photons_per_s_e2e": p.Nphoton / tot,
                     "steps_per_photon": rs[0].stats["steps"] / p.Nphoton}
    out["cpu_baseline"] = cpu_baseline(p, seconds_target=5.0, name="2D square")
    out["value"] = out["fp64"]["photons_per_s_e2e"]
    print(json.dumps(out), flush=True)
    return 0


def bench_batch(args):
    """64 cubes (20-80 mm edges, 48k-3.07M tets each, ~46M in all) with their own optics and
    pencil sources, photons log-uniform 1e5-1e7, in one persistent launch with the autotuned
    launch shape, plain and through a CUDA graph."""
    import valomc_gb300 as V
    from valomc_gb300 import meshgen as mg
    t0 = time.time()
    probs = mg.config_batch(count=64, photon_scale=args.batch_photon_scale)
    t_gen = time.time() - t0
    t0 = time.time()
    meshes = [V.Mesh(p) for p in probs]
    t_mesh = time.time() - t0
    tets = sum(p.Ne for p in probs)
    photons = sum(p.Nphoton for p in probs)
    t0 = time.time()
    tuned = V.autotune(meshes, probs, budget_s=6.0)
    t_tune = time.time() - t0
    res = {}
    for graph in (False, True):
        o = V.options(block_size=tuned.block_size, blocks_per_sm=tuned.blocks_per_sm, fetch_chunk=tuned.fetch_chunk,
                      use_graph=graph)
        _, st = V.run_batch(meshes, probs, opts=o)
        res["graph" if graph else "plain"] = {"kernel_s": st["seconds_kernel"], "wall_s": st["seconds_total"],
                                              "photons_per_s": photons / st["seconds_kernel"],
                                              "tet_steps_per_s": st["steps"] / st["seconds_kernel"],
                                              "steps_per_photon": st["steps"] / photons}
    dflt, st = V.run_batch(meshes, probs)
    res["untuned_photons_per_s"] = photons / st["seconds_kernel"]
    out = {"metric": "photons/s, 64 batched instances in one persistent launch", "unit": "photons/s",
           "value": res["graph"]["photons_per_s"], "instances": len(probs), "tets": tets, "photons": photons,
           "tuned": {"block_size": tuned.block_size, "blocks_per_sm": tuned.blocks_per_sm,
                     "fetch_chunk": tuned.fetch_chunk, "tune_s": t_tune},
           "mesh_gen_s": t_gen, "mesh_upload_s": t_mesh,
           "device_mesh_bytes": int(sum(m.device_bytes for m in meshes)), **res,
           "config": {"workload": "64 cubes L~logU[20,80] mm, pencil sources, config-4 optics",
                      "photon_scale": args.batch_photon_scale}}
    print(json.dumps(out), flush=True)
    return 0


def bench_serve(args):
    """Poisson request stream over 8 resident cubes (50k-2M tets), cosinic-disk or Gaussian
    sources at random top points, config-4 optics, photons log-uniform 1e5-1e7."""
    import valomc_gb300 as V
    from valomc_gb300 import meshgen as mg
    mix = mg.ServingMix(seed=5)
    meshes = [V.Mesh(b) for b in mix.base]
    srv = V.Server(max_slots=args.serve_slots, memory_budget=16 << 30, epoch_photons=int(args.serve_epoch),
                   block_size=args.serve_block)
    ids = [srv.add_mesh(m) for m in meshes]
    # warm the kernels and graphs
    k, p = mix.request()
    srv.wait(srv.submit(ids[k], p.copy(Nphoton=10000)))
    rng = np.random.default_rng(55)
    t0 = time.time()
    t, sub = 0.0, []
    while True:
        t += rng.exponential(1.0 / args.serve_rate)
        if t > args.serve_window:
            break
        k, p = mix.request()
        now = time.time() - t0
        if t > now:
            time.sleep(t - now)
        sub.append((srv.submit(ids[k], p), p.Nphoton))
    t_sub = time.time() - t0
    lat, ph, steps = [], 0, 0
    for rid, n in sub:
        r = srv.wait(rid)
        lat.append(r.stats["seconds_total"])
        ph += n
        steps += r.stats["steps"]
    wall = time.time() - t0
    srv.close()
    offered = sum(n for _, n in sub) / args.serve_window
    quarter = max(1, len(lat) // 4)
    q_first, q_last = float(np.median(lat[:quarter])), float(np.median(lat[-quarter:]))
    out = {"metric": "serve p50/p99 latency and photons/s", "unit": "s", "rate_hz": args.serve_rate,
           "window_s": args.serve_window, "epoch_photons": int(args.serve_epoch), "slots": args.serve_slots,
           "block_size": args.serve_block, "requests": len(sub),
           "submit_s": t_sub, "drain_s": wall - t_sub,
           "offered_photons_per_s": offered, "served_photons_per_s": ph / wall,
           "served_steps_per_s": steps / wall, "steps_per_photon": steps / max(ph, 1),
           # stable: the device keeps up (served >= 95% of offered) and the latency does not
           # grow over the window (median of the last quarter of requests vs the first)
           "stable": bool(ph / wall >= 0.95 * offered and q_last <= 2.0 * q_first + 0.05),
           "p50_first_quarter_s": q_first, "p50_last_quarter_s": q_last,
           "p50_s": float(np.percentile(lat, 50)), "p90_s": float(np.percentile(lat, 90)),
           "p99_s": float(np.percentile(lat, 99)), "value": float(np.percentile(lat, 99)),
           "config": {"workload": "8 cubes 50k-2M tets, cosinic disk / gaussian sources, photons logU[1e5,1e7]"}}
    print(json.dumps(out), flush=True)
    return 0


def matched_error(V, p, dev, B=10, n=400000):
    """chi2/dof of per-element batch means, FP32 form vs FP64 form, same photon count."""
    def bm(prec, base):
        xs = np.stack([V.run(p, precision=prec, device=dev, nphoton=n, seed=base + b).ER for b in range(B)])
        return xs.mean(0), xs.std(0, ddof=1) / math.sqrt(B), np.all(xs > 0, axis=0)
    m32, s32, h32 = bm(V.VMC_FP32, 100)
    m64, s64, h64 = bm(V.VMC_FP64, 900)
    hit = h32 & h64
    z = (m32[hit] - m64[hit]) / np.sqrt(s32[hit] ** 2 + s64[hit] ** 2)
    # ratio of FP32 error to the noise floor: sqrt of the mean squared z over 1 for an
    # unbiased estimator whose noise equals the FP64 form's
    rel32 = np.median(s32[hit] / m32[hit])
    rel64 = np.median(s64[hit] / m64[hit])
    return {"chi2_per_dof": float(np.mean(z ** 2)), "frac_within_3sigma": float(np.mean(np.abs(z) < 3)),
            "elements": int(hit.sum()), "noise_ratio_fp32_over_fp64": float(rel32 / rel64),
            "batches": B, "photons_per_batch": n}


if __name__ == "__main__":
    sys.exit(main())
