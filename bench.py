"""Benchmark of the photon-propagation path, every workload of the brief in one line.

Headline (the JSON line's value): the 60x60x30 mm inclusion phantom (648 000 tetrahedra,
1 mm grid, Gaussian sigma = 1 mm direct source, Fresnel boundary).  A step is one
simulation of ``--photons`` photons (default 1e8) through the FP32 tracking form with the
mesh resident on the device.

  value        photons/s with the mesh resident (per step: the job's setup and upload, the
               kernel and the read-back), max over ranks
  e2e          photons/s through vmc_run with host buffers: setup, uploads, kernel and the
               read-back of all results inside the timed region
  roofline     the pool kernel's algorithmic gather bytes (108 B per CW element step) over
               its CUDA-event duration, against the measured HBM copy bandwidth; the kernel
               is bound by instruction issue, with the measured L2 dependent-gather ceiling
               as its memory ceiling (l2_gather_frac), and runs at the SIMT efficiency of
               the committed ncu profile
  cpu_baseline the reference engine itself (MonteCarlo() of cpp/3d/MC3D.hpp, built with
               the reference's own flags -O3 -DUSE_OMP -fopenmp) on all host cores, on a
               bounded sample of the same workload; the CPU oracle where it is not built
  fp64         the plain FP64 form on the same workload
  matched_error  per-element error of each GPU form against the FP64 CPU oracle, as the
               ratio to the Monte Carlo noise floor (1 = no error beyond the noise)
  configs      the other workloads: the 2D square (plain FP64 and FP32, against the
               reference's 2D engine), the frequency-domain phantom, 64 batched instances in
               one persistent launch, and the serving loop at 50 requests/s
The L2 (129 MB) is flushed between timed steps by writing a 512 MB buffer.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
    python bench.py --config fd|batch|serve|square2d     (one workload, one line)
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_STEP_CW = 108  # element nodes 16 + coordinates 48 + HN row 16 + optics 12 + ER RMW 16
BYTES_PER_STEP_FD = 128  # + k 4 + EI RMW 16
METRIC = "photons/s FP32-track vs FP64 GPU at matched fluence error; serve p50/p99 latency"
WORKLOAD = "inclusion phantom 60x60x30 mm, 648000 tets, gaussian sigma 1 mm direct source, CW"
REF_BIN = os.path.join(ROOT, "oracle", "_ref")


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

    def _reduce(self, v, op):
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=op)
        return float(t.item())

    def max(self, v):
        return self._reduce(v, self.td.ReduceOp.MAX if self.ws > 1 else None)

    def sum(self, v):
        return self._reduce(v, self.td.ReduceOp.SUM if self.ws > 1 else None)

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


def ncu_profile():
    """DRAM bytes per element step, threads per warp instruction and issue activity of the
    FP32 pool kernel, from the committed ncu summary (profiles/)."""
    path = os.path.join(ROOT, "profiles", "pool_kernel_fp32_phantom.json")
    if os.path.exists(path):
        with open(path) as fp:
            return json.load(fp)
    return {}


# ---------------------------------------------------------------------------------------
# CPU side: the reference engine itself where it is built, else the oracle
# ---------------------------------------------------------------------------------------

def reference_binary(dim):
    path = os.path.join(REF_BIN, "ref3d_time" if dim == 3 else "ref2d_time")
    return path if os.path.exists(path) else None


class CpuBaseline:
    """Times MonteCarlo() on the host's cores on bounded samples of a workload: the
    reference's own engine (kind "reference") where oracle/_ref was built from the
    reference tree, else the oracle (the restatement, kind "port")."""

    def __init__(self, p, name, threads=None):
        self.p, self.name = p, name
        self.threads = threads or os.cpu_count() or 1
        self.exe = reference_binary(p.dim)
        self.kind = "reference" if self.exe else "port"
        self.tmp = None
        self.files = {}

    def _input(self, n):
        from valomc_gb300 import meshgen
        if n not in self.files:
            if self.tmp is None:
                self.tmp = tempfile.TemporaryDirectory()
            path = os.path.join(self.tmp.name, f"in_{n}.txt")
            meshgen.write_input(path, self.p.copy(Nphoton=n, seed=777))
            self.files[n] = path
        return self.files[n]

    def run(self, n):
        """Seconds of MonteCarlo() for n photons and the element steps (None for the engine)."""
        if self.exe:
            out = subprocess.run([self.exe, self._input(n), "-", str(self.threads)], capture_output=True, text=True,
                                 check=True).stdout.split()
            return float(out[out.index("seconds") + 1]), None
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        oracle.build()
        r = oracle.run(self.p, rng=oracle.RNG_MT, nthreads=self.threads, nphoton=n, seed=777, normalize=False)
        return r.seconds, r.steps

    def size_for(self, seconds):
        probe = max(self.threads * 200, 2000)
        s, _ = self.run(probe)
        return int(min(max(probe / max(s, 1e-6) * seconds, probe), 2e7))

    def describe(self, n, s):
        src = "cpp/3d/MC3D.hpp" if self.p.dim == 3 else "cpp/2d/MC2D.hpp"
        who = (f"the reference's MonteCarlo() ({src}, -O3 -DUSE_OMP -fopenmp)" if self.kind == "reference"
               else "the CPU oracle (the reference's algorithm restated, MT19937)")
        return {"value": n / s, "unit": "photons/s", "cores": self.threads, "kind": self.kind,
                "sample": f"{n} photons of the {self.name} workload, {who}, {self.threads} OpenMP threads, "
                          f"{s:.1f} s of MonteCarlo()"}


def reference_arm(args):
    """The reference's CPU implementation of the path on all host cores, each step a
    bounded sample of the phantom workload (rank 0 only)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from valomc_gb300 import meshgen as mg
    p = mg.config_3d_phantom(nphoton=1, seed=12345)
    cb = CpuBaseline(p, "phantom")
    steps = args.warmup + args.steps
    n = cb.size_for(max(2.0, args.ref_budget / steps))
    secs = []
    for i in range(steps):
        s, _ = cb.run(n)
        if i >= args.warmup:
            secs.append(s)
    t = float(np.mean(secs))
    v = n / t
    base = cb.describe(n, t)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "photons/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "photons_per_step": n},
            "cpu_baseline": base,
            "e2e": {"value": v, "unit": "photons/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------
# matched error: each GPU form against the FP64 CPU oracle, per element
# ---------------------------------------------------------------------------------------

def _welch(g, r, sel):
    Bg, Br = len(g), len(r)
    gm, gv = g.mean(0)[sel], g.var(0, ddof=1)[sel] / Bg
    rm, rv = r.mean(0)[sel], r.var(0, ddof=1)[sel] / Br
    s2 = gv + rv
    t = (gm - rm) / np.sqrt(s2)
    nu = s2 ** 2 / (gv ** 2 / (Bg - 1) + rv ** 2 / (Br - 1))
    return t, nu


def welch_error_to_noise(gpu_rows, ref_rows, null_rows, rel=0.05):
    """Over elements whose batch means have a relative standard error below `rel` on every
    side: chi2/dof of the Welch t statistics of the GPU batches against the oracle's, and
    against independent GPU batches of the oracle's size (the noise floor: the value the
    comparison takes when the GPU form is distributed exactly as the oracle), and
    error_to_noise = sqrt(chi2 / chi2 of the noise floor).  chi2/dof of an exact match
    exceeds the t-expectation mean(nu / (nu - 2)) because batch means of tallies are
    skewed; both are reported."""
    from scipy.stats import t as student_t
    g, r, n = np.asarray(gpu_rows), np.asarray(ref_rows), np.asarray(null_rows)
    ok = np.all(g != 0, axis=0) & np.all(r != 0, axis=0) & np.all(n != 0, axis=0)
    for x in (g, r, n):
        ok[ok] &= x.std(0, ddof=1)[ok] / math.sqrt(len(x)) < rel * np.abs(x.mean(0)[ok])
    t, nu = _welch(g, r, ok)
    tn, _ = _welch(g, n, ok)
    chi2, chi2n = float(np.mean(t * t)), float(np.mean(tn * tn))
    q = student_t.ppf(0.5 + 0.99730020393674 / 2, nu)
    return {"elements": int(ok.sum()), "chi2_per_dof": chi2, "noise_floor_chi2_per_dof": chi2n,
            "t_expectation": float(np.mean(nu / (nu - 2))), "error_to_noise": math.sqrt(chi2 / chi2n),
            "frac_within_3sigma": float(np.mean(np.abs(t) < q)), "mean_t": float(np.mean(t))}


def matched_error(V, p, dev, B=10, n_ref=100_000):
    """B batches of the FP64 CPU oracle (MT19937, all host cores) against B batches of each
    GPU form (both forms at the same photon count per batch), with B more GPU batches of
    the oracle's size for the noise floor."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    t0 = time.time()
    ref = []
    for b in range(B):
        r = oracle.run(p, rng=oracle.RNG_MT, nthreads=os.cpu_count() or 1, nphoton=n_ref, seed=60000 + 1000 * b)
        ref.append(np.concatenate([r.ER, r.EBR]))
    t_ref = time.time() - t0
    out = {"reference": f"FP64 CPU oracle, {B} batches x {n_ref} photons (MT19937, {os.cpu_count()} threads, "
                        f"{t_ref:.1f} s)", "batches": B}
    for prec, name, n in ((V.VMC_FP32, "fp32", 400_000), (V.VMC_FP64, "fp64", 400_000)):
        mesh = V.Mesh(p, precision=prec, device=dev)

        def rows(count, seed0):
            res = [V.run_batch([mesh], [p.copy(Nphoton=count, seed=seed0 + b)], precision=prec, device=dev)[0][0]
                   for b in range(B)]
            return [np.concatenate([x.ER, x.EBR]) for x in res]

        out[name] = welch_error_to_noise(rows(n, 100), ref, rows(n_ref, 500))
        out[name]["photons_per_batch"] = n
        mesh.close()
    out["fp32_over_fp64_error"] = out["fp32"]["error_to_noise"] / out["fp64"]["error_to_noise"]
    return out


# ---------------------------------------------------------------------------------------
# the other workloads
# ---------------------------------------------------------------------------------------

def run_fd(args, dev=0):
    """The frequency-domain phantom (per-tet lognormal mua, U(8, 12) mus, 100 MHz): both forms."""
    import valomc_gb300 as V
    from valomc_gb300 import meshgen as mg
    p = mg.config_3d_fd(nphoton=int(args.photons), seed=12345)
    out = {"workload": "FD phantom 648000 tets, f = 100 MHz, lognormal mua, U(8,12) mus"}
    for prec, name, n, reps in ((V.VMC_FP32, "fp32", int(args.photons), max(1, min(args.steps, 3))),
                                (V.VMC_FP64, "fp64", int(args.fd_fp64_photons), 1)):
        mesh = V.Mesh(p, precision=prec, device=dev)
        q = p.copy(Nphoton=n)
        V.run_batch([mesh], [q.copy(Nphoton=min(n, 1_000_000))], precision=prec, device=dev)
        ks, st = [], None
        for _ in range(reps):
            flush_l2()
            _, st = V.run_batch([mesh], [q], precision=prec, device=dev)
            ks.append(st["seconds_kernel"])
        k = float(np.median(ks))
        out[name] = {"photons": n, "photons_per_s": n / k, "tet_steps_per_s": st["steps"] / k,
                     "steps_per_photon": st["steps"] / n, "achieved_gbs_128B_per_step": BYTES_PER_STEP_FD * st["steps"] / k / 1e9}
        mesh.close()
    out["fp32_over_fp64"] = out["fp32"]["photons_per_s"] / out["fp64"]["photons_per_s"]
    return out


def run_square2d(args, dev=0):
    """The 2D square (10x10 mm, 200 triangles, cosinic source on edges 4..7, 1e6 photons):
    both forms through vmc_run (host buffers), and the reference's 2D engine on all host
    cores."""
    import valomc_gb300 as V
    from valomc_gb300 import meshgen as mg
    p = mg.config_2d_square(nphoton=1_000_000, seed=12345)
    out = {"workload": "10x10 mm square, 200 triangles, cosinic edges 4-7, 1e6 photons"}
    for prec, name in ((V.VMC_FP64, "fp64"), (V.VMC_FP32, "fp32")):
        V.run(p, precision=prec, device=dev)
        rs = [V.run(p, precision=prec, device=dev) for _ in range(max(1, min(args.steps, 5)))]
        k = float(np.median([r.stats["seconds_kernel"] for r in rs]))
        tot = float(np.median([r.stats["seconds_total"] for r in rs]))
        out[name] = {"photons_per_s_kernel": p.Nphoton / k, "photons_per_s_e2e": p.Nphoton / tot,
                     "steps_per_photon": rs[0].stats["steps"] / p.Nphoton}
    cb = CpuBaseline(p, "2D square")
    s, _ = cb.run(p.Nphoton)
    out["cpu_baseline"] = cb.describe(p.Nphoton, s)
    for name in ("fp64", "fp32"):
        out[name]["e2e_over_cpu"] = out[name]["photons_per_s_e2e"] / out["cpu_baseline"]["value"]
    return out


def run_batch_config(args, dev=0):
    """64 cubes (20-80 mm edges, 48k-3.07M tets each, ~60M in all) with their own optics and
    pencil sources, photons log-uniform 1e5-1e7, in one persistent launch with the autotuned
    launch shape, plain and through a CUDA graph."""
    import valomc_gb300 as V
    from valomc_gb300 import meshgen as mg
    t0 = time.time()
    probs = mg.config_batch(count=64, photon_scale=args.batch_photon_scale)
    t_gen = time.time() - t0
    t0 = time.time()
    meshes = [V.Mesh(p, device=dev) for p in probs]
    t_mesh = time.time() - t0
    tets = sum(p.Ne for p in probs)
    photons = sum(p.Nphoton for p in probs)
    t0 = time.time()
    tuned = V.autotune(meshes, probs, budget_s=args.tune_budget)
    t_tune = time.time() - t0
    res = {}
    for graph in (False, True):
        o = V.options(block_size=tuned.block_size, blocks_per_sm=tuned.blocks_per_sm, fetch_chunk=tuned.fetch_chunk,
                      refill_lanes=tuned.refill_lanes, use_graph=graph, device=dev)
        _, st = V.run_batch(meshes, probs, opts=o)
        res["graph" if graph else "plain"] = {"kernel_s": st["seconds_kernel"], "wall_s": st["seconds_total"],
                                              "photons_per_s": photons / st["seconds_kernel"],
                                              "tet_steps_per_s": st["steps"] / st["seconds_kernel"],
                                              "steps_per_photon": st["steps"] / photons}
    _, st = V.run_batch(meshes, probs, device=dev)
    res["untuned_photons_per_s"] = photons / st["seconds_kernel"]
    for m in meshes:
        m.close()
    return {"workload": "64 cubes L~logU[20,80] mm, pencil sources, config-4 optics, one persistent launch",
            "photons_per_s": res["graph"]["photons_per_s"], "instances": len(probs), "tets": tets, "photons": photons,
            "tuned": {"block_size": tuned.block_size, "blocks_per_sm": tuned.blocks_per_sm,
                      "fetch_chunk": tuned.fetch_chunk, "refill_lanes": tuned.refill_lanes, "tune_s": t_tune},
            "mesh_gen_s": t_gen, "mesh_upload_s": t_mesh, **res, "photon_scale": args.batch_photon_scale}


def run_serve(args, dev=0):
    """Poisson request stream at --serve-rate over 8 resident cubes (50k-2M tets),
    cosinic-disk or Gaussian sources at random top points, config-4 optics, photons
    log-uniform 1e5-1e7, for --serve-window seconds; then the same requests submitted at
    once (the loop's capacity for this mix).  --serve-samples > 1 adds further samples of
    the same stream (other requests and arrival times on the same meshes), summarised in
    `other_samples`: one 10 s sample's offered load varies by several percent around the
    stream's mean."""
    import copy
    import valomc_gb300 as V
    from valomc_gb300 import meshgen as mg
    mix = mg.ServingMix(seed=5)
    meshes = [V.Mesh(b, device=dev) for b in mix.base]
    rng0 = copy.deepcopy(mix.rng)

    def server():
        srv = V.Server(max_slots=args.serve_slots, memory_budget=16 << 30, epoch_photons=int(args.serve_epoch),
                       block_size=args.serve_block, device=dev, slicing=args.serve_slicing,
                       epoch_max_ms=args.serve_epoch_max_ms)
        return srv, [srv.add_mesh(m) for m in meshes]

    def sample(seed):
        # seed 0: the default sample; k > 0: the same meshes, other requests and arrivals
        mix.rng = copy.deepcopy(rng0) if seed == 0 else np.random.default_rng(1000 + seed)
        srv, ids = server()
        k, p = mix.request()
        srv.wait(srv.submit(ids[k], p.copy(Nphoton=10000)))  # warm the kernels and graphs
        rng = np.random.default_rng(55 + seed)
        T = args.serve_window
        t0 = time.time()
        t, sub = 0.0, []
        while True:
            t += rng.exponential(1.0 / args.serve_rate)
            if t > T:
                break
            k, p = mix.request()
            now = time.time() - t0
            if t > now:
                time.sleep(t - now)
            sub.append((srv.submit(ids[k], p), p.Nphoton, time.time() - t0, k, p))
        t_sub = time.time() - t0
        lat, fin, ph, steps = [], [], 0, 0
        for rid, n, ts, _, _ in sub:
            r = srv.wait(rid)
            lat.append(r.stats["seconds_total"])
            fin.append(ts + r.stats["seconds_total"])
            ph += n
            steps += r.stats["steps"]
        wall = time.time() - t0
        srv.close()
        n_sub = np.array([x[1] for x in sub], float)
        t_in = np.array([x[2] for x in sub])
        fin = np.array(fin)
        lat = np.array(lat)
        offered = n_sub.sum() / T
        # steady state: the last three quarters of the window (the first is the start-up from
        # an empty device); the photons of requests that finished in it, against those offered
        lo = T / 4
        served_steady = n_sub[(fin >= lo) & (fin <= T)].sum() / (T - lo)
        offered_steady = n_sub[(t_in >= lo) & (t_in <= T)].sum() / (T - lo)
        q = max(1, len(lat) // 4)
        q2, q4 = float(np.median(lat[q:2 * q])), float(np.median(lat[-q:]))
        out = {"sample": seed, "requests": len(sub), "submit_s": t_sub, "drain_s": wall - t_sub,
               "offered_photons_per_s": offered, "served_photons_per_s_incl_drain": ph / wall,
               "offered_photons_per_s_steady": offered_steady, "served_photons_per_s_steady": served_steady,
               "served_steps_per_s": steps / wall, "steps_per_photon": steps / max(ph, 1),
               # stable: in the steady part of the window the device serves >= 95% of what is
               # offered, and the latency does not grow (median of the last quarter of requests
               # at most twice the second quarter's, plus 50 ms)
               "stable": bool(served_steady >= 0.95 * offered_steady and q4 <= 2.0 * q2 + 0.05),
               "p50_second_quarter_s": q2, "p50_last_quarter_s": q4,
               "p50_s": float(np.percentile(lat, 50)), "p90_s": float(np.percentile(lat, 90)),
               "p99_s": float(np.percentile(lat, 99)),
               "p50_small_s": float(np.median(lat[n_sub < 1e6])) if (n_sub < 1e6).any() else None}
        return out, sub, n_sub

    out, sub, n_sub = sample(args.serve_seed)
    out = {"workload": "8 cubes 50k-2M tets, cosinic disk / gaussian sources, photons logU[1e5,1e7]",
           "rate_hz": args.serve_rate, "window_s": args.serve_window, "slicing": args.serve_slicing,
           "epoch_max_ms": args.serve_epoch_max_ms,
           # the mix's mean request is 1e5..1e7 log-uniform: (1e7 - 1e5) / ln(100) photons
           "offered_expected_photons_per_s": args.serve_rate * (1e7 - 1e5) / math.log(100.0), **out}
    if args.serve_capacity:
        srv, ids = server()
        srv.wait(srv.submit(ids[sub[0][3]], sub[0][4].copy(Nphoton=10000)))
        t0 = time.time()
        rids = [srv.submit(ids[x[3]], x[4]) for x in sub]
        for r in rids:
            srv.wait(r)
        out["capacity_photons_per_s"] = n_sub.sum() / (time.time() - t0)
        srv.close()
    keys = ("sample", "offered_photons_per_s", "offered_photons_per_s_steady", "served_photons_per_s_steady",
            "stable", "p50_second_quarter_s", "p50_last_quarter_s", "p50_s", "p99_s")
    others = []
    for k in range(1, args.serve_samples):
        o, _, _ = sample(args.serve_seed + k)
        others.append({key: o[key] for key in keys})
    if others:
        out["other_samples"] = others
    for m in meshes:
        m.close()
    return out


# ---------------------------------------------------------------------------------------
# the headline
# ---------------------------------------------------------------------------------------

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--photons", type=float, default=1e8)
    ap.add_argument("--fp64-photons", type=float, default=1e7)
    ap.add_argument("--fd-fp64-photons", type=float, default=2e6)
    ap.add_argument("--ref-budget", type=float, default=100.0, help="seconds of reference work in --impl reference")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-extras", action="store_true", help="the headline numbers only (profiling runs)")
    ap.add_argument("--config", default="all", choices=["all", "phantom", "fd", "batch", "serve", "square2d"],
                    help="all: the headline line with every workload; phantom: the headline alone; "
                         "fd / batch / serve / square2d: one workload, one line")
    ap.add_argument("--batch-photon-scale", type=float, default=1.0)
    ap.add_argument("--tune-budget", type=float, default=6.0)
    ap.add_argument("--serve-rate", type=float, default=50.0)
    ap.add_argument("--serve-window", type=float, default=10.0)
    ap.add_argument("--serve-epoch", type=float, default=0.0,
                    help="photons per serving epoch (0: the loop's own choice by backlog)")
    ap.add_argument("--serve-slots", type=int, default=64, help="requests the serving loop simulates at once")
    ap.add_argument("--serve-block", type=int, default=0, help="threads per CTA of the serving launches (0: default)")
    ap.add_argument("--serve-slicing", type=int, default=0,
                    help="serving slices: 0 the server's default, 1 water-filling, 2 shortest remaining first")
    ap.add_argument("--serve-samples", type=int, default=2,
                    help="samples of the request stream: the default one, then others on the same meshes")
    ap.add_argument("--serve-seed", type=int, default=0,
                    help="0: the default sample of requests and arrivals; k > 0: another sample")
    ap.add_argument("--serve-epoch-max-ms", type=int, default=0,
                    help="cap of the serving loop's epochs, ms of work (0: the server's default)")
    ap.add_argument("--serve-capacity", type=int, default=1, help="1: also time the same requests submitted at once")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    single = {"fd": run_fd, "batch": run_batch_config, "serve": run_serve, "square2d": run_square2d}
    if args.config in single:
        out = single[args.config](args)
        out["config"] = args.config
        print(json.dumps(out), flush=True)
        return 0

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

    if rank == 0:
        peak, peak_kind = measured_peaks()
        achieved = BYTES_PER_STEP_CW * steps_per_launch / kmean / 1e9
        prof = ncu_profile()
        dram_per_step = prof.get("dram_bytes_per_step")
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
            # the kernel is bound by instruction issue (ncu: issue-active, threads per warp
            # instruction); its memory ceiling is the L2 dependent-gather rate, since the
            # mesh stays in L2; frac is against the HBM copy peak as the contract has it
            "roofline": {"bound": "issue", "memory_ceiling": "l2_gather", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": (dram_per_step * steps_per_launch) if dram_per_step else None,
                         "algorithmic_bytes_per_launch": BYTES_PER_STEP_CW * steps_per_launch,
                         "simt_threads_per_inst": prof.get("threads_per_inst"),
                         "issue_active": prof.get("issue_active"),
                         "profile": prof.get("kernel")},
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
            cb = CpuBaseline(p, "phantom")
            n_cpu = cb.size_for(args.cpu_seconds)
            s, _ = cb.run(n_cpu)
            line["cpu_baseline"] = cb.describe(n_cpu, s)
            line["cpu_baseline"]["gpu_over_cpu"] = value / line["cpu_baseline"]["value"]
            line["cpu_baseline"]["e2e_over_cpu"] = e2e_value / line["cpu_baseline"]["value"]
            mesh.close()
            line["configs"] = {}
            for name, fn in (("square2d", run_square2d), ("fd", run_fd), ("batch", run_batch_config),
                             ("serve", run_serve)):
                t0 = time.time()
                line["configs"][name] = fn(args, dev)
                line["configs"][name]["bench_s"] = time.time() - t0
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
