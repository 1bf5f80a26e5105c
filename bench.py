"""Benchmark of the GB300 BEM hot path: served BEM solves per second on the 0.6 m relief.

Workload (one step = one BEM solve): 0.6 x 0.6 x 0.05 m box whose top face is a 64 x 64 grid
displaced by a seeded 64 x 64 uniform [0, 0.1] m heightmap smoothed with sigma = 2 cells
(20480 triangles); 2 kHz; normal plane-wave incidence; 181 receivers on a 5 m semicircle;
cluster leaf 32, admissibility factor 2; ACA tolerance 1e-4; BiCGSTAB to 1e-6 relative residual.
A solve is: H-matrix assembly (near-field quadrature + ACA), BiCGSTAB (mixed: complex FP32
H-matrix with FP64 dots and FP64 iterative refinement), receiver far field.

  value : served solves/s: the request server with --slots slots (default 4) and the mesh
          registered (resident) before the timed region; --steps requests of this workload are
          submitted at once and timed with CUDA events bracketing a device-wide synchronisation.
          Slots overlap one request's assembly with another's solve. p50/p99: request latency
          under Poisson arrivals at half the saturated rate.
  e2e   : solves/s through the reference-facing C-ABI call (ac3d_set_points + ac3d_pressures,
          DiffBEM.pvals) from pinned host buffers, one request after another, host<->device
          copies inside the timed region.
  single_context: one context, one request after another, inputs resident (ac3d_pressures_dev).
The H-matrix of one solve (~550 MB) is larger than L2, so no L2 flush is needed between steps.

--impl reference times the FP64 CPU restatement of the reference algorithm (oracle/) on the
host cores on the same workload: each timed step is one full solve (mesh, assembly, BiCGSTAB,
receivers); the untimed warm-up steps assemble only.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "served BEM solves/sec + p50/p99 latency, FP32+refine vs FP64 GPU at 1e-6 resid"
UNIT = "solves/s"
FREQ = 2000.0
LEAF, FACTOR, ACA_TOL, SOLVER_TOL = 32, 2.0, 1e-4, 1e-6
DIRECTION = (0.0, -1.0, 0.0)
RESTART = 300  # GMRES basis: iterations per cycle
WORKLOAD = ("0.6 m relief, 64x64 smoothed seeded heightmap, 20480 triangles, 2 kHz, normal plane wave, "
            "181 receivers on a 5 m semicircle, leaf 32, eta 2, ACA 1e-4, BiCGSTAB 1e-6")


# the reference pipeline's third-octave bands (acoustics_pipeline.py:7), 3 frequencies each
SWEEP_BANDS = (100, 125, 160, 200, 250, 315, 400, 500, 630, 800, 1000, 1250, 1600, 2000, 2500, 3150, 4000)
SWEEP_WORKLOAD = ("served sweep: 0.6 m reliefs (30x7x30 box, subdiv_top {subdivs}: {sizes} triangles), seeded "
                  "smoothed 64x64 heightmap, 3 frequencies per third-octave band 100 Hz - 4 kHz (51 per relief), "
                  "normal plane wave, 181 receivers on a 5 m semicircle, leaf 32, eta 2, ACA 1e-4, BiCGSTAB 1e-6")


def band_frequencies(band: float, n: int = 3):
    """n log-spaced frequencies over +-1/6 octave around a band centre (get_frequencies,
    helpers.cpp:67-83)."""
    bw = 2.0 ** (1.0 / 6.0)
    return list(np.exp(np.linspace(np.log(band / bw), np.log(band * bw), n)))


def sweep_workload(seed: int, subdivs):
    from acoustic_reliefs_gb300 import meshes
    hm = meshes.smooth_heightmap(64, seed)
    reliefs = [meshes.relief(0.6, 0.6, 0.05, 30, 7, 30, s, hm) for s in subdivs]
    freqs = [f for b in SWEEP_BANDS for f in band_frequencies(b)]
    reqs = [(m, f) for m in range(len(reliefs)) for f in freqs]
    order = np.random.default_rng(seed).permutation(len(reqs))
    return reliefs, [reqs[i] for i in order]


def run_served(precision, reliefs, reqs, Ls, slots, rate, seed, krylov="gmres"):
    """Submits the requests with Poisson arrivals at `rate` per second (all at once if rate is None)
    to a server with `slots` slots; returns (solves/s over the makespan, latencies ms, results)."""
    import threading
    from acoustic_reliefs_gb300.serve import Server
    with Server(slots=slots, precision=precision, krylov=krylov, restart=RESTART) as srv:
        ids = [srv.add_mesh(R.Ps, R.Es, LEAF, FACTOR, ACA_TOL, SOLVER_TOL)[0] for R in reliefs]
        # one untimed request per mesh (kernel set-up, allocator warm-up, footprint estimates)
        for mid in ids:
            srv.wait(srv.submit(mid, 1000.0, Ls, ("plane", DIRECTION)))
        gaps = (np.random.default_rng(seed + 1).exponential(1.0 / rate, size=len(reqs)) if rate
                else np.zeros(len(reqs)))
        handles = [None] * len(reqs)
        t_sub = [0.0] * len(reqs)

        def feeder():
            t_next = time.perf_counter()
            for i, (m, f) in enumerate(reqs):
                t_next += gaps[i]
                dt = t_next - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                t_sub[i] = time.perf_counter()
                handles[i] = srv.submit(ids[m], f, Ls, ("plane", DIRECTION))

        th = threading.Thread(target=feeder)
        th.start()
        th.join()
        res = [srv.wait(h) for h in handles]
    done = [t_sub[i] + res[i][1]["latency_ms"] / 1e3 for i in range(len(reqs))]
    makespan = max(done) - min(t_sub)
    lat = [r[1]["latency_ms"] for r in res]
    return len(reqs) / makespan, lat, res


def served_sweep(args, Ls):
    subdivs = tuple(int(x) for x in args.sweep_subdivs.split(","))
    reliefs, reqs = sweep_workload(0, subdivs)
    out = {"workload": SWEEP_WORKLOAD.format(subdivs="/".join(map(str, subdivs)),
                                             sizes="/".join(str(len(R.Es)) for R in reliefs)),
           "requests": len(reqs), "slots": args.slots}
    thr, lat_sat, res_m = run_served("mixed", reliefs, reqs, Ls, args.slots, None, 0, args.krylov)
    out["mixed"] = {"solves_per_s": thr, "offered": "all requests at t=0 (saturated)",
                    "p50_ms_saturated": float(np.percentile(lat_sat, 50)),
                    "p99_ms_saturated": float(np.percentile(lat_sat, 99))}
    rate = 0.5 * thr
    thr_l, lat_l, _ = run_served("mixed", reliefs, reqs, Ls, args.slots, rate, 0, args.krylov)
    out["mixed"].update({"poisson_rate_per_s": rate, "solves_per_s_at_rate": thr_l,
                         "p50_ms": float(np.percentile(lat_l, 50)), "p99_ms": float(np.percentile(lat_l, 99))})
    info = [r[1] for r in res_m]
    out["mixed"].update({
        "run_ms_p50": float(np.percentile([i["run_ms"] for i in info], 50)),
        "run_ms_p99": float(np.percentile([i["run_ms"] for i in info], 99)),
        "ms_graph_mean": float(np.mean([i["ms_graph"] for i in info])),
        "note": "saturated latency = queueing + run; run_ms = admitted to result; ms_graph = host time capturing "
                "and instantiating the request's solver graphs"})
    if not args.no_fp64_sweep:
        thr64, lat64, res_d = run_served("fp64", reliefs, reqs, Ls, args.slots, None, 0, args.krylov)
        errs = [float(np.linalg.norm(a[0] - b[0]) / np.linalg.norm(b[0])) for a, b in zip(res_m, res_d)]
        out["fp64"] = {"solves_per_s": thr64, "offered": "all requests at t=0 (saturated)",
                       "p50_ms_saturated": float(np.percentile(lat64, 50)),
                       "p99_ms_saturated": float(np.percentile(lat64, 99))}
        out["speedup_mixed_over_fp64"] = thr / thr64
        out["max_pressure_rel_err_mixed_vs_fp64"] = max(errs)
        out["requests_above_1e-4"] = int(sum(e > 1e-4 for e in errs))
        out["max_pressure_rel_err_by_relief"] = {
            str(len(R.Es)): max(e for e, (mi, _) in zip(errs, reqs) if mi == i) for i, R in enumerate(reliefs)}
    out["max_rel_residual"] = max(r[1]["rel_residual"] for r in res_m)
    return out


def gradient_leg():
    """The multi-incidence gradient at full size: 0.9 m relief with a 128 x 128 heightmap (81024
    triangles, 37445 differentiable heights), 1, 2 and 4 kHz, 37 incidence angles in the xy plane,
    receivers on a 10 m semicircle: loss = 1 - mean coefficient and its gradient in one call,
    timed once after a small warm-up call."""
    from acoustic_reliefs_gb300 import meshes
    from acoustic_reliefs_gb300.acoustics3d import DiffBEM
    R = meshes.relief(0.9, 0.9, 0.05, 48, 7, 48, 2, meshes.smooth_heightmap(128, 0))
    th = np.radians(np.linspace(-90.0, 90.0, 37))
    dirs = np.stack([np.sin(th), -np.cos(th), np.zeros_like(th)], 1)
    freqs = [1000.0, 2000.0, 4000.0]
    x = np.random.default_rng(4).uniform(0.0, 0.01, size=len(R.diff_pts))
    bem = DiffBEM(LEAF, FACTOR, [1000.0], 1, ACA_TOL, ACA_TOL, SOLVER_TOL, precision="mixed")
    bem.silent = True
    bem.set_krylov("gmres", RESTART)
    bem.set_listeners(meshes.semicircle(10.0, 181))
    bem.precompute(R.Ps, R.Es, R.diff_pts)
    bem.gradient_multi(x, [1000.0], dirs[:2])
    t0 = time.perf_counter()
    loss, g, cf = bem.gradient_multi(x, freqs, dirs)
    dt = time.perf_counter() - t0
    st = bem.stats()
    return {"workload": "0.9 m relief, 128x128 smoothed seeded heightmap, 81024 triangles, 37445 heights; 1/2/4 kHz x "
                        "37 plane-wave angles (-90..90 deg in the xy plane); 181 receivers on a 10 m semicircle; "
                        "loss 1 - mean coefficient; mixed precision, GMRES, leaf 32, eta 2, ACA 1e-4, tol 1e-6",
            "seconds": dt, "gradients_per_s": 1.0 / dt, "loss": loss, "grad_norm": float(np.linalg.norm(g)),
            "solves": st["solves"], "iterations": st["iterations"], "ms_assemble": st["ms_assemble"],
            "ms_solve": st["ms_solve"], "ms_adjoint": st["ms_adjoint"],
            "note": "per frequency one H-matrix: forward and transposed block solves (16 directions per block), "
                    "shape-derivative terms of 16 directions per derivative evaluation (ac3d_gradient_multi)"}


def product_call_leg():
    """The reference pipeline's own forward call (acoustics_pipeline.py:7,11-17) on its submitted
    0.6 m relief (the 38686-triangle mesh held in tests/golden/ref_relief_cat.npz): DiffBEM(128, 1.5,
    17 third-octave bands 100 Hz - 4 kHz, 3 frequencies each, ACA and solver tolerances 1e-5, point
    source at (0, 100, 0), 1297-point hemisphere of radius 50 m), every band's diffusion coefficient
    in one values() call (51 solves), with the drop-in's defaults (mixed precision, BiCGSTAB as the
    reference, exact receiver product) and with GMRES; timed after a one-band warm-up call."""
    from acoustic_reliefs_gb300.acoustics3d import DiffBEM
    g = np.load(os.path.join(ROOT, "tests", "golden", "ref_relief_cat.npz"))
    bands = [float(b) for b in SWEEP_BANDS]
    out = {"workload": "reference product call: DiffBEM(128, 1.5, 17 bands 100 Hz - 4 kHz, 3, 1e-5, 1e-5, 1e-5, "
                       "(0, 100, 0), 50, 5) on the reference's submitted 0.6 m relief (38686 triangles), values()"}
    for krylov in ("bicgstab", "gmres"):
        bem = DiffBEM(128, 1.5, bands, 3, 1e-5, 1e-5, 1e-5, (0.0, 100.0, 0.0), 50, 5)
        bem.silent = True
        bem.set_krylov(krylov, RESTART)
        bem.set_mesh(g["Ps"], g["Es"])
        bem.band_value(1000.0)
        t0 = time.perf_counter()
        cs = bem.values()
        dt = time.perf_counter() - t0
        st = bem.stats()
        out[krylov] = {"seconds": dt, "solves": 3 * len(bands), "solves_per_s": 3 * len(bands) / dt,
                       "iterations": st["iterations"], "ms_assemble": st["ms_assemble"], "ms_solve": st["ms_solve"],
                       "coef_1000": cs[bands.index(1000.0)],
                       "coef_1000_minus_oracle": cs[bands.index(1000.0)] - float(g["coef_1000"])}
    return out


def block_c5_leg():
    """The large block solve: 0.9 m relief with a 256 x 256 heightmap (210240 triangles) at 4
    kHz, 16 plane-wave directions as one block; error against the FP64 solve of the first
    direction."""
    from acoustic_reliefs_gb300 import meshes
    from acoustic_reliefs_gb300.acoustics3d import DiffBEM
    R = meshes.relief(0.9, 0.9, 0.05, 40, 7, 40, 3, meshes.smooth_heightmap(256, 0))
    Ls = meshes.semicircle(5.0, 181)
    rng = np.random.default_rng(1)
    dirs = rng.normal(size=(16, 3))
    dirs[:, 1] = -np.abs(dirs[:, 1]) - 0.5
    dirs[0] = DIRECTION
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    bem = DiffBEM(LEAF, FACTOR, [4000.0], 1, ACA_TOL, ACA_TOL, SOLVER_TOL, precision="mixed")
    bem.silent = True
    bem.set_krylov("gmres", RESTART)
    bem.set_mesh(R.Ps, R.Es)
    t0 = time.perf_counter()
    P = bem.pvals_multi(4000.0, dirs, Ls)
    dt = time.perf_counter() - t0
    st = bem.stats()
    mv_ms, mv_bytes = bem.block_matvec_timing(16, 10)
    bem.set_tensor_cores(False)
    mv_ms_cc, _ = bem.block_matvec_timing(16, 10)
    bem.set_tensor_cores(True)
    b64 = DiffBEM(LEAF, FACTOR, [4000.0], 1, ACA_TOL, ACA_TOL, SOLVER_TOL, precision="fp64",
                  incident=("plane", dirs[0]))
    b64.silent = True
    b64.set_krylov("gmres", RESTART)
    b64.set_mesh(R.Ps, R.Es)
    t1 = time.perf_counter()
    y64 = b64.pvals(4000.0, Ls)
    dt64 = time.perf_counter() - t1
    peak, _ = measured_peak()
    gbs = mv_bytes / (mv_ms / 1e3) / 1e9
    return {"workload": "0.9 m relief, 256x256 smoothed seeded heightmap, 210240 triangles, 4 kHz, 16 plane-wave "
                        "directions as one block, 181 receivers on a 5 m semicircle, leaf 32, eta 2, ACA 1e-4, tol 1e-6",
            "seconds_per_block": dt, "solves_per_s": 16 / dt, "hmat_bytes": st["hmat_bytes"],
            "ms_assemble": st["ms_assemble"], "ms_solve": st["ms_solve"], "iterations": st["iterations"],
            "near_entries": st["near_entries"], "lr_entries": st["lr_entries"],
            "block_matvec_ms": mv_ms, "block_matvec_bytes": int(mv_bytes), "block_matvec_gbs": gbs,
            "block_matvec_frac_of_hbm": gbs / peak, "block_matvec_ms_cuda_cores": mv_ms_cc,
            "dot_pass": "tensor cores (tcgen05.mma kind::tf32 from the segments split once into TF32 hi/lo tiles: "
                        "hi*hi + hi*lo + lo*hi in two MMAs per K step, FP32 accumulation in tensor memory); "
                        "gather and reduce passes on the CUDA cores",
            "fp64_single_solve_s": dt64,
            "pressure_rel_err_vs_fp64": float(np.linalg.norm(P[0] - y64) / np.linalg.norm(y64))}


def workload(seed: int = 0):
    from acoustic_reliefs_gb300 import meshes
    R = meshes.relief_20k(seed)
    return R, meshes.semicircle(5.0, 181)


def dist_init(backend=None):
    """Replica ranks from the torchrun environment: NCCL on GPU machines (one GPU per rank), gloo
    otherwise. Replicas exchange only the timing maximum, never data."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = backend or ("nccl" if torch.cuda.is_available() else "gloo")
        if backend == "nccl":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, units_per_rank: int, ms_max: float) -> float:
    """Units all replicas processed per second of the slowest replica's time."""
    return world * units_per_rank / (ms_max / 1e3)


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join("/tmp", f"ac3d_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        try:
            self.f.close()
        except Exception:
            pass

    def summary(self):
        try:
            rows = [l.strip().split(",") for l in open(self.path) if l.strip()]
        except OSError:
            rows = []
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and "Active" in r[5 + i] and "Not" not in r[5 + i]:
                    reasons.add(n)
        busy = [v for v in sm if v > 0.5 * max(sm)] if sm else []
        return {"sm_mhz": float(np.median(busy)) if busy else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peak():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def measured_traffic(krylov):
    """DRAM bytes of one matvec of this workload, in the variant the solver runs, from the
    committed ncu capture summarised in profiles/traffic.json (None if absent)."""
    try:
        d = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        return int(d["matvec"][krylov]["traffic_bytes"]), d["matvec"][krylov]["command"]
    except (OSError, KeyError, ValueError):
        return None, None


def cpu_baseline_sample(R, Ls, threads=None):
    """One full FP64 solve by the oracle (the reference algorithm restated in C++/OpenMP)."""
    import oracle
    if threads:
        oracle.lib().orc_set_threads(int(threads))
    cores = oracle.lib().orc_num_threads()
    k = oracle.wavenumber(FREQ)
    t0 = time.perf_counter()
    m = oracle.Mesh(R.Ps, R.Es, LEAF, FACTOR)
    y, x, info = oracle.solve_pressures(m, k, DIRECTION, 1, Ls, ACA_TOL, ACA_TOL, SOLVER_TOL, listener="aca")
    dt = time.perf_counter() - t0
    return dt, cores, y, info


def reference_warmup(R):
    """Untimed warm-up step of the reference arm: mesh and H-matrix assembly by the oracle (page-in
    of the code and the OpenMP pool; a full solve takes half a minute)."""
    import oracle
    m = oracle.Mesh(R.Ps, R.Es, LEAF, FACTOR)
    oracle.HMat(m, oracle.wavenumber(FREQ), ACA_TOL)


def run_reference(args):
    # rank 0 alone times the CPU reference on the host cores; the other ranks exit without work
    # (no process group: the ranks exchange nothing)
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    R, Ls = workload(0)
    for _ in range(args.warmup):
        reference_warmup(R)
    times, iters = [], []
    cores = 0
    for _ in range(args.steps):
        dt, cores, _, info = cpu_baseline_sample(R, Ls)  # one full solve per timed step
        times.append(dt)
        iters.append(int(info["iters"]))
    total = sum(times)
    v = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": WORKLOAD, "l2": "inputs larger than L2"},
        "p50_ms": 1e3 * float(np.percentile(times, 50)), "p99_ms": 1e3 * float(np.percentile(times, 99)),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"per timed step one full FP64 solve of this workload by the oracle restatement "
                                   f"(mesh, H-matrix assembly, BiCGSTAB to 1e-6 in {iters[0]} iterations, ACA "
                                   f"receivers), OpenMP over {cores} threads; warm-up steps: mesh and assembly only; "
                                   f"the reference itself does not build here (empty Eigen submodule)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def served_c2(args, R, Ls, precision, n_req, n_warm, rate=None, seed=0, clocks=None, krylov=None):
    """Requests of this workload (one mesh, 2 kHz) through the request server with args.slots slots.
    rate None: all n_req requests submitted at once, timed with CUDA events bracketing a device-wide
    synchronisation on both sides (the server's slots run on their own streams); else Poisson
    arrivals at `rate` per second. Returns (solves/s, ms, latencies ms, kernel launches, results)."""
    import threading
    import torch
    from acoustic_reliefs_gb300 import _lib as _L
    from acoustic_reliefs_gb300.serve import Server
    lib = _L.lib()
    inc = ("plane", DIRECTION)
    with Server(slots=args.slots, precision=precision, krylov=krylov or args.krylov, restart=RESTART) as srv:
        mid = srv.add_mesh(R.Ps, R.Es, LEAF, FACTOR, ACA_TOL, SOLVER_TOL)[0]
        for _ in range(n_warm):  # one at a time, then a full round of slots
            srv.wait(srv.submit(mid, FREQ, Ls, inc))
        for h in [srv.submit(mid, FREQ, Ls, inc) for _ in range(args.slots)]:
            srv.wait(h)
        gaps = np.random.default_rng(seed + 1).exponential(1.0 / rate, size=n_req) if rate else np.zeros(n_req)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        l0 = lib.ac3d_kernel_launches()
        ctx = clocks if clocks is not None else _NullCtx()
        with ctx:
            e0.record()
            handles = [None] * n_req

            def feeder():
                t_next = time.perf_counter()
                for i in range(n_req):
                    t_next += gaps[i]
                    dt = t_next - time.perf_counter()
                    if dt > 0:
                        time.sleep(dt)
                    handles[i] = srv.submit(mid, FREQ, Ls, inc)

            th = threading.Thread(target=feeder)
            th.start()
            th.join()
            res = [srv.wait(h) for h in handles]
            torch.cuda.synchronize()
            e1.record()
            e1.synchronize()
        launches = lib.ac3d_kernel_launches() - l0
    ms = e0.elapsed_time(e1)
    lat = [r[1]["latency_ms"] for r in res]
    return n_req / (ms / 1e3), ms, lat, launches, res


class _NullCtx:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def run_single(args):
    """One context on one stream, one solve after another, no request-server threads: the command
    line for kernel captures under a profiler. Prints the single-context rate, the solver
    statistics and the matvec timing of the last solve's H-matrix."""
    import torch
    torch.cuda.set_device(0)
    from acoustic_reliefs_gb300.acoustics3d import DiffBEM
    R, Ls = workload(0)
    bem = DiffBEM(LEAF, FACTOR, [FREQ], 1, ACA_TOL, ACA_TOL, SOLVER_TOL, precision="mixed",
                  incident=("plane", DIRECTION), device=0)
    bem.silent = True
    bem.set_solver(0, args.inner_tol, 10)
    bem.set_krylov(args.krylov, RESTART)
    bem.set_mesh(R.Ps, R.Es)
    dev = torch.device("cuda", 0)
    L = len(Ls)
    Ls_dev = torch.tensor(Ls, dtype=torch.float64, device=dev)
    out = torch.zeros(2 * L, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        bem.pvals_dev(FREQ, out.data_ptr(), Ls_dev.data_ptr(), L, stream.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        bem.pvals_dev(FREQ, out.data_ptr(), Ls_dev.data_ptr(), L, stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    st = bem.stats()
    mv_ms, mv_bytes = bem.matvec_timing(20)
    print(json.dumps({"mode": "single context (kernel captures)", "workload": WORKLOAD, "krylov": args.krylov,
                      "solves_per_s": args.steps / (ms / 1e3), "ms_per_solve": ms / args.steps,
                      "iterations": st["iterations"], "refinement_steps": st["outer_steps"],
                      "rel_residual": st["rel_residual"], "ms_assemble": st["ms_assemble"],
                      "ms_solve": st["ms_solve"], "matvec_ms": mv_ms, "matvec_bytes": int(mv_bytes)}), flush=True)
    return 0


def block_dirs(n):
    """n seeded plane-wave directions from the upper half space, the first the headline's."""
    rng = np.random.default_rng(1)
    dirs = rng.normal(size=(n, 3))
    dirs[:, 1] = -np.abs(dirs[:, 1]) - 0.5
    dirs[0] = DIRECTION
    return dirs / np.linalg.norm(dirs, axis=1, keepdims=True)


def run_single_block(args):
    """One context, one block solve after another (16 directions on the 20k relief at 2 kHz, the
    multi_rhs leg's workload): the command line for captures of the block-matvec kernels."""
    from acoustic_reliefs_gb300.acoustics3d import DiffBEM
    R, Ls = workload(0)
    bem = DiffBEM(LEAF, FACTOR, [FREQ], 1, ACA_TOL, ACA_TOL, SOLVER_TOL, precision="mixed")
    bem.silent = True
    bem.set_krylov(args.krylov, RESTART)
    bem.set_mesh(R.Ps, R.Es)
    dirs = block_dirs(max(args.multi_rhs, 1))
    for _ in range(args.warmup):
        bem.pvals_multi(FREQ, dirs, Ls)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bem.pvals_multi(FREQ, dirs, Ls)
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    st = bem.stats()
    mv_ms, mv_bytes = bem.block_matvec_timing(16, 10)
    print(json.dumps({"mode": "single context, block solves (kernel captures)", "rhs": len(dirs),
                      "ms_per_block": 1e3 * dt, "iterations": st["iterations"], "block_matvec_ms": mv_ms,
                      "block_matvec_bytes": int(mv_bytes)}), flush=True)
    return 0


def run_gpu(args):
    import torch
    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    from acoustic_reliefs_gb300.acoustics3d import DiffBEM
    R, Ls = workload(rank)
    dev = torch.device("cuda", local)

    def make(prec):
        b = DiffBEM(LEAF, FACTOR, [FREQ], 1, ACA_TOL, ACA_TOL, SOLVER_TOL, precision=prec,
                    incident=("plane", DIRECTION), device=local)
        b.silent = True
        b.set_solver(0, args.inner_tol, 10)
        b.set_krylov(args.krylov, RESTART)
        b.set_mesh(R.Ps, R.Es)
        return b

    # ---- headline: served solves/s (args.slots slots, all requests at once), mesh resident
    barrier(world)
    clk = ClockSampler(local)
    value, total_ms, lat_sat, launches, res_m = served_c2(args, R, Ls, "mixed", args.steps, args.warmup, clocks=clk)
    total_ms = max_over_ranks(world, total_ms)
    value = whole_job_rate(world, args.steps, total_ms)
    barrier(world)
    # latency under a sustainable load: Poisson arrivals at half the saturated rate
    rate = 0.5 * value / world
    thr_p, _, lat_p, _, _ = served_c2(args, R, Ls, "mixed", args.steps, 1, rate=rate, seed=rank)

    # ---- one context, one request at a time (device-resident mesh and receivers)
    bem = make("mixed")
    L = len(Ls)
    Ls_dev = torch.tensor(Ls, dtype=torch.float64, device=dev)
    out = torch.zeros(2 * L, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(b):
        b.pvals_dev(FREQ, out.data_ptr(), Ls_dev.data_ptr(), L, stream.cuda_stream)

    for _ in range(args.warmup):
        step(bem)
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    for i in range(args.steps):
        step(bem)
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    lat1 = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]
    single_ms = max_over_ranks(world, evs[0].elapsed_time(evs[-1]))
    st = bem.stats()
    y_mixed = out.cpu().numpy().view(np.complex128).copy()
    single = {"solves_per_s": world * args.steps / (single_ms / 1e3), "ms_per_solve": single_ms / args.steps,
              "p50_ms": float(np.percentile(lat1, 50)), "p99_ms": float(np.percentile(lat1, 99)),
              "note": "one context, requests one after another, mesh and receivers resident (ac3d_pressures_dev)"}
    served_equal = all(np.array_equal(r[0], y_mixed) for r in res_m)

    # assembly throughput of the last step: 6 kernel evaluations per near-field entry and per
    # entry ACA evaluated (every row and column of every pass, the dropped converging term included)
    evals = 6 * (st["near_entries"] + st["aca_entries_evaluated"])
    assembly = {"ms": st["ms_assemble"], "near_entries": st["near_entries"],
                "aca_entries_evaluated": st["aca_entries_evaluated"], "kernel_evaluations": int(evals),
                "kernel_evaluations_per_s": evals / (st["ms_assemble"] / 1e3),
                "stored_gbs": 8 * (st["near_entries"] + st["lr_entries"]) / (st["ms_assemble"] / 1e3) / 1e9,
                "arithmetic": "double-float (about 47 bits) on the FP32 pipes, FP32 storage",
                "note": "near field, ACA (two streams), packing; one context"}

    # roofline of the dominant kernel (H-matrix matvec) on the last step's H-matrix
    mv_ms, mv_bytes = bem.matvec_timing(50)
    peak, peak_kind = measured_peak()
    achieved = mv_bytes / (mv_ms / 1e3) / 1e9

    # end to end through the reference-facing C-ABI call (DiffBEM.pvals): pinned host mesh points and
    # receivers in, pressures out, every step
    Ps_h = torch.tensor(R.Ps, dtype=torch.float64).pin_memory().numpy()
    Ls_h = torch.tensor(Ls, dtype=torch.float64).pin_memory().numpy()
    y_h = torch.zeros(2 * L, dtype=torch.float64).pin_memory().numpy()
    from acoustic_reliefs_gb300 import _lib as _L
    lib = _L.lib()

    def e2e_step():
        bem._check(lib.ac3d_set_points(bem._h, _L.ptr(Ps_h)))
        bem._check(lib.ac3d_pressures(bem._h, FREQ, _L.ptr(Ls_h), L, _L.ptr(y_h)))

    e2e_step()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(world, time.perf_counter() - t0)
    e2e_value = world * args.steps / e2e_s

    # the plain FP64 GPU path on the same workload, served the same way
    n64 = max(2, args.steps // 2)
    f64_value, f64_ms, _, _, res_d = served_c2(args, R, Ls, "fp64", n64, 1)
    f64_ms = max_over_ranks(world, f64_ms)
    f64_value = world * n64 / (f64_ms / 1e3)
    y64 = res_d[0][0]
    err64 = float(np.linalg.norm(y_mixed - y64) / np.linalg.norm(y64))
    it64 = res_d[0][1]["iterations"]

    # the reference's solver (BiCGSTAB) served the same way, for comparison with the headline
    bicg = None
    if args.krylov != "bicgstab":
        bicg = {"note": "BiCGSTAB (the reference's solver) inner solves, request server with the same slots"}
        for prec, nreq, nwarm in (("mixed", args.steps, args.warmup), ("fp64", n64, 1)):
            _, bms, _, _, res_b = served_c2(args, R, Ls, prec, nreq, nwarm, krylov="bicgstab")
            bms = max_over_ranks(world, bms)
            bicg[prec] = {"solves_per_s": world * nreq / (bms / 1e3), "ms_per_step": bms / nreq,
                          "iterations": res_b[0][1]["iterations"],
                          "pressure_rel_err_vs_headline": float(np.linalg.norm(res_b[0][0] - y_mixed) /
                                                                np.linalg.norm(y_mixed))}

    # block solve: 16 incidence directions of the same frequency against one H-matrix
    multi = None
    if args.multi_rhs > 0:
        dirs = block_dirs(args.multi_rhs)
        bem.pvals_multi(FREQ, dirs, Ls)  # warm-up
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            P = bem.pvals_multi(FREQ, dirs, Ls)
        dt = (time.perf_counter() - t0) / reps
        stm = bem.stats()
        multi = {"solves_per_s": args.multi_rhs / dt, "ms_per_block": 1e3 * dt, "rhs": args.multi_rhs,
                 "block_iterations": stm["iterations"], "refinement_steps": stm["outer_steps"],
                 "max_rel_residual": stm["rel_residual"],
                 "pressure_rel_err_vs_single_solve": float(np.linalg.norm(P[0] - y_mixed) / np.linalg.norm(y_mixed)),
                 "note": "host API call (ac3d_solve_multi), assembly + block solve + receivers per block; "
                         + ("one GMRES cycle per direction sharing each block matvec" if args.krylov == "gmres"
                            else "block BiCGSTAB")}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        dt, cores, ycpu, info = cpu_baseline_sample(R, Ls)
        cpu = {"value": 1.0 / dt, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"one full FP64 solve of this workload by the oracle restatement ({dt:.1f} s: assembly, "
                         f"BiCGSTAB {info['iters']} iterations to 1e-6, ACA receivers), OpenMP over {cores} threads",
               "err_vs_gpu_mixed": float(np.linalg.norm(y_mixed - ycpu) / np.linalg.norm(ycpu))}

    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 storage/products, f64 dots+refinement",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "precision": "mixed (FP32 + FP64 refinement)",
                   "krylov": (f"GMRES({RESTART}) cycles, two classical Gram-Schmidt passes in FP32, inside the FP64 "
                              "refinement loop" if args.krylov == "gmres" else "BiCGSTAB (as the reference)"),
                   "serving": f"request server, {args.slots} slots, {args.steps} requests submitted at once; "
                              "mesh registered (resident) before the timed region",
                   "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (H-matrix ~550 MB per solve)"},
        "p50_ms": float(np.percentile(lat_p, 50)), "p99_ms": float(np.percentile(lat_p, 99)),
        "latency": {"poisson_rate_per_s": rate, "solves_per_s_at_rate": thr_p,
                    "p50_ms": float(np.percentile(lat_p, 50)), "p99_ms": float(np.percentile(lat_p, 99)),
                    "p50_ms_saturated": float(np.percentile(lat_sat, 50)),
                    "p99_ms_saturated": float(np.percentile(lat_sat, 99)),
                    "note": "p50/p99 at the top level are request latencies (submit to result on the host) under "
                            "Poisson arrivals at half the saturated rate; saturated = all requests at once"},
        "single_context": single,
        "bicgstab": bicg,
        "served_results_bitwise_equal_to_single_context": bool(served_equal),
        "fp64_gpu": {"value": f64_value, "unit": UNIT, "ms_per_step": f64_ms / n64, "requests": n64,
                     "serving": f"request server, {args.slots} slots, all requests at once",
                     "speedup_mixed_over_fp64": value / f64_value, "pressure_rel_err_mixed_vs_fp64": err64,
                     "iterations": it64},
        "solve": {"iterations": st["iterations"], "refinement_steps": st["outer_steps"],
                  "rel_residual": st["rel_residual"], "ms_assemble": st["ms_assemble"], "ms_solve": st["ms_solve"],
                  "ms_listener": st["ms_listener"], "near_entries": st["near_entries"],
                  "lr_entries": st["lr_entries"], "mean_rank": st["mean_rank"], "max_rank": st["max_rank"],
                  "hmat_bytes": st["hmat_bytes"]},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(Ps_h.nbytes + Ls_h.nbytes),
                "d2h_bytes_per_step": int(y_h.nbytes),
                "path": "DiffBEM C-ABI (ac3d_set_points + ac3d_pressures), one request after another"},
        "assembly": assembly,
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": measured_traffic(args.krylov)[0],
                     "traffic_source": "profiles/traffic.json: " + str(measured_traffic(args.krylov)[1]),
                     "kernel": "H-matrix matvec (dot + reduce + gather passes)",
                     "bytes_per_launch": int(mv_bytes), "ms_per_launch": mv_ms, "peak_kind": peak_kind},
        "clocks": clk.summary(),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if multi:
        line["multi_rhs"] = multi
    if args.sweep_subdivs not in ("", "none") and world == 1:
        line["served_sweep"] = served_sweep(args, Ls)
    if not args.no_gradient_leg and world == 1:
        line["gradient_c4"] = gradient_leg()
    if not args.no_c5_leg and world == 1:
        line["block_c5"] = block_c5_leg()
    if not args.no_product_leg and world == 1:
        try:
            line["product_call"] = product_call_leg()
        except Exception as e:  # an extra leg: its failure is reported, not fatal to the line
            line["product_call"] = {"error": f"{type(e).__name__}: {e}"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--inner-tol", type=float, default=1e-6)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sweep-subdivs", default="0,1,2,3",
                    help="subdiv_top levels of the served sweep ('none' to skip; 5280/10680/32280/118680 triangles)")
    ap.add_argument("--slots", type=int, default=4, help="server slots (concurrent requests)")
    ap.add_argument("--no-fp64-sweep", action="store_true")
    ap.add_argument("--no-gradient-leg", action="store_true", help="skip the 81k-triangle 37-angle gradient")
    ap.add_argument("--no-c5-leg", action="store_true", help="skip the 210k-triangle 16-direction block solve")
    ap.add_argument("--no-product-leg", action="store_true",
                    help="skip the reference pipeline's own call (17 bands on its 38686-triangle relief)")
    ap.add_argument("--product-call-only", action="store_true",
                    help="only the reference pipeline's own call (one JSON object)")
    ap.add_argument("--multi-rhs", type=int, default=16, help="directions of the block-solve leg (0 to skip)")
    ap.add_argument("--krylov", default="gmres", choices=["gmres", "bicgstab"],
                    help="inner solver of every GPU leg (BiCGSTAB is the reference's; a served BiCGSTAB leg is "
                         "reported beside a GMRES headline)")
    ap.add_argument("--single-context", action="store_true",
                    help="only one context on one stream (no request server): the command for kernel captures")
    ap.add_argument("--single-block", action="store_true",
                    help="one context, block solves of --multi-rhs directions: the command for block-kernel captures")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.single_block:
        return run_single_block(args)
    if args.single_context:
        return run_single(args)
    if args.product_call_only:
        print(json.dumps({"product_call": product_call_leg()}), flush=True)
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
