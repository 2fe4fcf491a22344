"""Benchmark of the MBIR ICD hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload ...]

Default workload: bright-field (BF) reconstruction of a 512 x 256 x 128 (x, y, z) volume from 61
views over +-60 deg at 2 deg on a 512 x 256 detector: 200 ellipsoid nanoparticles on a slab,
seeded synthetic Poisson counts at 1e4 electrons with +-3% per-view dose drift (the engine
takes -log itself).  A step is one NHICD equivalent iteration: 20 updateVoxels calls (10 on
homogeneous 1/20 line lists, 10 on the non-homogeneous top-1/20 lists), i.e. about one sweep's
worth of voxel updates.  HAADF workloads (one step = one full ICD sweep) remain selectable.

Metric: voxel updates per second = voxels updated in the timed steps / ICD device time
(zero-skipped visits are reported beside it, not counted).

Timing: W untimed warm-up steps, then K steps whose ICD kernels are bracketed by CUDA events on
the engine's launching stream (the engine accumulates them); before every timed step a 512 MiB
buffer is written to flush the 129 MB L2.  `e2e` runs the same workload through the public C
ABI from host buffers: upload of the tilt series, set-up and forward projection, calls with
offset and variance updates, and read-back of the volume, all inside the timed region.
`--impl reference` times the reference algorithm (the FP64 oracle restatement of the
reference's multi-threaded CPU path) on all host cores on a bounded sample of the workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "openmbir-tem_gb300")
ORACLE = os.path.join(ROOT, "oracle")
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402

WORKLOADS = {
    # name: (modality, n_r, n_t, thickness_nm, max_deg, step_deg, particles)
    "bf-512x256x128-61v": ("BF", 512, 256, 64.0, 60.0, 2.0, 200),
    "haadf-512x256x128-61v": ("HAADF", 512, 256, 64.0, 60.0, 2.0, 200),
    "haadf-128x32x64-71v": ("HAADF", 128, 32, 32.0, 70.0, 2.0, 0),
}
DEFAULT_WORKLOAD = "bf-512x256x128-61v"
METRIC = "ICD voxel-updates/s"
CALLS_PER_EQUIT = 20  # k_NumNonHomogeniousIter: updateVoxels calls per equivalent iteration


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_data(name, seed=0, n_t_override=None):
    import synthetic
    mod, n_r, n_t, th, mx, st, npart = WORKLOADS[name]
    if n_t_override:
        n_t = n_t_override
    if mod == "BF":
        y, ang = synthetic.bf_particles_on_slab(n_r=n_r, n_t=n_t, thickness=th, max_deg=mx,
                                                step_deg=st, n_particles=npart, seed=seed)
    elif npart == 0:
        y, ang, _ = synthetic.haadf_two_spheres(n_r=n_r, n_t=n_t, max_deg=mx, step_deg=st,
                                                seed=seed)
    else:
        y, ang, _ = synthetic.particles_on_slab(n_r=n_r, n_t=n_t, thickness=th, max_deg=mx,
                                                step_deg=st, n_particles=npart, seed=seed)
    return y, ang, th, mod


def params_for(mbir, th, mod, outer=20, inner=1):
    if mod == "BF":
        p = mbir.default_params(mbir.BF)
        p.sigma_x = 0.02
        p.use_default_offset = 1
        p.default_dosage = 1.0e4
        p.bragg_threshold = 5.0e10  # Bragg rejection off, as the workload runs it
    else:
        p = mbir.default_params()
        p.sigma_x = 0.2
    p.sample_thickness = th
    p.diffuseness = 0.1
    p.num_resolutions = 1
    p.outer_iterations = outer
    p.inner_iterations = inner
    p.stop_threshold = 0.0
    return p


def oracle_params_for(th, mod):
    """The same workload parameters as params_for, for the CPU restatement alone: the reference
    arm and the CPU baseline never load the product library."""
    sys.path.insert(0, ORACLE)
    import oracle
    o = oracle.OrcParams()
    o.delta_xz_factor = 1.0
    o.interpolate_factor = 1.0
    o.length_z = th
    o.extend_object = 0
    o.x_shrink_factor = 0.6
    o.z_stretch = 2
    o.response_bins = 64
    o.profile_resolution = 1536
    o.beam_resolution = 512
    o.compat_double_angle = 0 if mod == "BF" else 1
    o.sigma_x = 0.02 if mod == "BF" else 0.2
    o.mrf_p = 2.0
    o.mrf_q = 1.1
    o.mrf_c = 0.01 if mod == "BF" else 0.001
    o.mrf_alpha = 1.5
    o.target_gain = 1.0
    o.default_variance = 1.0
    o.use_default_offset = 1 if mod == "BF" else 0
    o.default_offset = -np.log(1.0e4) if mod == "BF" else 0.0
    o.joint_estimation = 1
    o.noise_model = 0 if mod == "BF" else 1
    o.zero_skipping = 1
    o.stop_threshold = 0.0
    o.outer_iterations = 20
    o.inner_iterations = 1
    o.threshold_reduction_factor = 1.0
    o.modality = 1 if mod == "BF" else 0
    o.noise_estimation = 1 if mod == "BF" else 0
    o.bragg_threshold = 5.0e10 if mod == "BF" else 0.0
    o.bragg_delta = 0.5
    o.nhicd = 1 if mod == "BF" else 0
    return o


def workload_config(name):
    """The workload as both arms report it (config is the same dict on the GPU line and on the
    reference line; measured details go elsewhere)."""
    mod, n_r, n_t, th, mx, st, npart = WORKLOADS[name]
    views = int(round(2 * mx / st)) + 1
    return {"workload": name, "modality": mod, "volume_zxy": [int(round(2 * th)), n_r, n_t],
            "views": views, "detector": [n_r, n_t],
            "step": ("one NHICD equivalent iteration (20 updateVoxels calls)" if mod == "BF"
                     else "one full ICD sweep"),
            "l2": "flushed before every timed step (512 MiB write)",
            "parallelism": "replicas"}


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
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

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() in ("active", "0x1", "1"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def cpu_reference_sample(name, budget_s=12.0, n_t=32, threads=None, max_calls=None):
    """The reference algorithm on the host cores: the oracle's restatement of the reference's
    CPU path (same arithmetic; y split into one contiguous range per worker as the reference's
    task split) on the workload's x-z geometry with n_t detector rows (n_t voxel slices), for
    about `budget_s` seconds of calls.  BF: NHICD calls (homogeneous and non-homogeneous lists
    alternating); HAADF: full sweeps.  Returns the cpu_baseline dict (voxel updates/s)."""
    sys.path.insert(0, ORACLE)
    import oracle
    threads = threads or os.cpu_count() or 1
    y, ang, th, mod = make_data(name, n_t_override=n_t)
    o = oracle.Oracle(oracle_params_for(th, mod), y, ang)
    o.prepare()
    upd = 0.0
    calls = 0
    t0 = time.perf_counter()
    if mod == "BF":
        nl = o.nz * o.nx
        perm = oracle.rand_list_perm(1, nl)
        master = np.empty(nl, np.int32)
        master[perm] = np.arange(nl, dtype=np.int32)
        n_el = nl // CALLS_PER_EQUIT
        while True:
            k = calls
            if k % 2 == 0:
                s = (k // 2) % CALLS_PER_EQUIT
                lines = master[s * n_el:(s + 1) * n_el]
            else:
                o.bf_vsc()
                lines = o.bf_nh_lines(o.bf_nh_threshold())
            upd += o.bf_sweep_lines_mt(lines, 0 if k == 0 else 1, 0, threads)[3]
            calls += 1
            if (max_calls and calls >= max_calls) or time.perf_counter() - t0 > budget_s:
                break
        what = f"{calls} NHICD calls"
    else:
        while True:
            upd += o.sweep_reference_mt(1, 0 if calls == 0 else 1, 0, threads)[3]
            calls += 1
            if (max_calls and calls >= max_calls) or time.perf_counter() - t0 > budget_s:
                break
        what = f"{calls} reference-order sweeps"
    dt = time.perf_counter() - t0
    return {"value": upd / dt, "unit": "voxel-updates/s", "cores": threads, "kind": "port",
            "sample": f"{o.nz}x{o.nx}x{o.ny} volume ({n_t} detector rows of the workload), "
                      f"{what}, FP64 oracle restatement of the reference's CPU path, "
                      f"{threads} threads, {dt:.1f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    t0 = time.perf_counter()
    budget = min(60.0, max(5.0, 4.0 * max(args.steps, 1)))
    res = cpu_reference_sample(args.workload, budget_s=budget)
    wall = time.perf_counter() - t0
    line = {"metric": METRIC, "value": res["value"], "unit": res["unit"], "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": workload_config(args.workload),
            "cpu_baseline": res,
            "e2e": {"value": res["value"], "unit": res["unit"], "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line))


# ---- batched and served forms ------------------------------------------------------------
def uneven_series(n, seed=0, large_frac=0.0, bf_frac=0.0):
    """n tilt series with the uneven sizes of the batched workload: N_x in U{128..512},
    N_y (detector rows) in U{16..256}, N_z in U{32..128}, views in U{41..141} over +-60..70 deg;
    a fraction `large_frac` takes the 512x256x128 / 61-view shape, `bf_frac` are bright field.
    Random ellipsoid phantoms, seeded noise.  Returns [(modality, counts, angles, thickness)]."""
    import synthetic
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        if rng.uniform() < large_frac:
            n_r, n_t, n_z, views, mx = 512, 256, 128, 61, 60.0
        else:
            n_r = int(rng.integers(128, 513))
            n_t = int(rng.integers(16, 257))
            n_z = int(rng.integers(32, 129))
            views = int(rng.integers(41, 142))
            mx = float(rng.uniform(60.0, 70.0))
        th = n_z / 2.0
        ang = np.linspace(-mx, mx, views)
        shapes = synthetic.random_ellipsoids(6, n_r, n_t, n_z, seed=int(rng.integers(1 << 30)),
                                             axes=(3.0, min(15.0, n_z / 4)))
        proj = np.zeros((views, n_r, n_t))
        t = -n_t / 2 + np.arange(n_t) + 0.5
        for sh in shapes:  # each ellipsoid projected onto the detector rows it covers
            rows = np.nonzero(np.abs(t - sh[1]) < sh[4])[0]
            if len(rows) == 0:
                continue
            lo, hi = rows[0], rows[-1] + 1
            off = -n_t / 2 + lo + (hi - lo) / 2
            sub = (sh[0], sh[1] - off, sh[2], sh[3], sh[4], sh[5], sh[6])
            proj[:, :, lo:hi] += synthetic.ellipsoid_projection(ang, n_r, hi - lo, [sub])
        if rng.uniform() < bf_frac:
            y, _ = synthetic.bf_counts(proj, seed=k)
            out.append(("BF", y, ang.astype(np.float32), th))
        else:
            y, _ = synthetic.haadf_measurements(proj, seed=k)
            out.append(("HAADF", y, ang.astype(np.float32), th))
    return out


def batch_measure(mbir, n, seed=1, batch_threads=None, tol=1e-4, max_outer=60):
    """Time to a relative cost tolerance for n uneven HAADF reconstructions: one at a time
    through the step-wise C ABI (sweep, gain/offset, variance, cost per outer iteration) against
    all of them advancing together in one persistent launch per sweep (mbir_batch_run)."""
    import torch
    data = uneven_series(n, seed=seed)

    def engine(item):
        mod, y, ang, th = item
        p = params_for(mbir, th, mod, outer=max_outer)
        p.lane_shape = 4 if y.shape[0] > 96 else (3 if y.shape[0] > 64 else 1)
        e = mbir.Engine(p)
        e.set_sinogram(y, ang)
        e.prepare()
        return e

    # one at a time
    seq_s, seq_upd, seq_iters = 0.0, 0.0, []
    phase = {"sweep_s": 0.0, "joint_estimation_s": 0.0, "variance_s": 0.0, "cost_s": 0.0}

    def timed(key, fn):
        t = time.perf_counter()
        r = fn()
        phase[key] += time.perf_counter() - t
        return r

    for item in data:
        with engine(item) as e:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            prev = None
            for it in range(max_outer):
                timed("sweep_s", lambda: e.sweep(it, 0))
                timed("joint_estimation_s", e.joint_estimation)
                timed("variance_s", e.update_weights)
                c = timed("cost_s", e.cost)[0]
                if prev is not None and abs(c - prev) <= tol * abs(c):
                    break
                prev = c
            seq_s += time.perf_counter() - t0
            seq_iters.append(it + 1)
            seq_upd += e.status().voxels_updated
    # all together
    engines = [engine(item) for item in data]
    with mbir.Batch(0) as b:
        if batch_threads:
            b.set_threads(batch_threads)
        for e in engines:
            b.add(e)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        iters, _ = b.run(max_outer, tol)
        bat_s = time.perf_counter() - t0
        bat_threads = b.threads()
        bat_sweep_s = b.total_ms() / 1e3
        bat_upd = sum(e.status().voxels_updated for e in engines)
    for e in engines:
        e.close()
    vox = sum(int(np.prod([d[1].shape[1], d[1].shape[2], 2 * d[3]])) for d in data)
    return {"speedup": seq_s / bat_s, "series": n, "voxels_total": vox, "tolerance": tol,
            "max_outer": max_outer,
            "sequential": {"wall_s": seq_s, "voxel_updates": seq_upd,
                           "voxel_updates_per_s": seq_upd / seq_s,
                           "outer_iterations": int(np.sum(seq_iters)), "phases": phase},
            "batched": {"wall_s": bat_s, "voxel_updates": bat_upd,
                        "sweep_device_s": bat_sweep_s,
                        "threads_per_cta": bat_threads,
                        "voxel_updates_per_s": bat_upd / bat_s,
                        "outer_iterations": int(np.sum(iters))}}


PRECISION_WORKLOAD = "precision-1024x512x256-121v"


def run_precision(args):
    """The precision study: the bright-field workload family at 1024 x 512 detector, 121 views
    over +-60 deg at 1 deg, volume 1024 x 512 x 256 (x, y, z), the particles-on-slab phantom at
    4x the areal particle density of the 512 x 256 workload.  Seeded synthetic data: the
    voxelised phantom projected by the engine's own FP32 projector, then Poisson counts at 1e4
    electrons with +-3% per-view dose drift.  The FP32 engine and the FP64 engine run the same
    20 NHICD calls (one equivalent iteration) with offset and variance updates from the same
    start, in the same visit order (the row walk, which the FP32 engine runs as dependency
    levels); the line reports each result's error of the FP32 run against the FP64 run after
    the first call (one call from the same state: the arithmetic alone) and after the 20 calls
    (where the non-homogeneous lines chosen from the update magnitudes can differ as well)."""
    import torch
    torch.cuda.set_device(0)
    import build as pkg_build
    pkg_build.build()
    import mbir
    import synthetic
    n_r, n_t, th, mx, st = 1024, 512, 128.0, 60.0, 1.0
    ang = synthetic.tilt_angles(mx, st).astype(np.float32)
    n_part = 4 * 200 * (n_r * n_t) // (512 * 256)
    t0 = time.perf_counter()
    ph = params_for(mbir, th, "HAADF", outer=1)
    with mbir.Engine(ph) as e:
        e.set_sinogram(np.ones((len(ang), n_r, n_t), np.float32), ang)
        nz, nx, ny = e.dims()[:3]
        vol = synthetic.particles_on_slab_volume(nx, ny, nz, th, n_part, seed=0)
        e.set_initial_volume(vol)
        e.prepare()
        proj = e.projection()
    del vol
    counts, _ = synthetic.bf_counts(proj, seed=1)
    del proj
    gen_s = time.perf_counter() - t0
    out = {}
    for calls in (1, CALLS_PER_EQUIT):
        for name, prec in (("fp32", mbir.FP32), ("fp64", mbir.FP64)):
            p = params_for(mbir, th, "BF", outer=calls, inner=1)
            p.precision = prec
            # the FP32 calls in the dependency levels of the row walk: the FP64 engine's own
            # visit order, so that the errors are those of the arithmetic alone
            p.call_schedule = 2
            with mbir.Engine(p) as e:
                e.set_sinogram(counts, ang)
                t = time.perf_counter()
                e.run()
                wall = time.perf_counter() - t
                s_ = e.status()
                g, off, var = e.nuisance()
                out[(calls, name)] = {
                    "volume": e.volume().astype(np.float64), "cost": e.cost()[0], "offset": off,
                    "variance": var, "wall_s": wall, "icd_ms": s_.icd_ms_total,
                    "calls": s_.sweeps_done, "staged": s_.staged,
                    "updated": int(s_.voxels_updated), "dims": [int(v) for v in e.dims()[:3]]}

    def rel(x, y):
        return float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))

    def errors(calls):
        a, b = out[(calls, "fp32")], out[(calls, "fp64")]
        return {"volume_rel_l2": rel(a["volume"], b["volume"]),
                "volume_max_abs": float(np.abs(a["volume"] - b["volume"]).max()),
                "volume_max": float(np.abs(b["volume"]).max()),
                "cost_rel": abs(a["cost"] - b["cost"]) / abs(b["cost"]),
                "offset_max_rel": float(np.max(np.abs(a["offset"] - b["offset"]) /
                                               np.abs(b["offset"]))),
                "variance_rel": float(np.max(np.abs(a["variance"] - b["variance"]) /
                                             np.abs(b["variance"]))),
                "voxels_updated": [a["updated"], b["updated"]]}

    a, b = out[(CALLS_PER_EQUIT, "fp32")], out[(CALLS_PER_EQUIT, "fp64")]
    line = {"metric": "FP32 vs FP64 error per result", "workload": PRECISION_WORKLOAD,
            "data": "synthetic (voxelised particles-on-slab phantom, engine projector, Poisson "
                    "counts)", "n_gpus": 1,
            "config": {"workload": PRECISION_WORKLOAD, "detector": [n_r, n_t], "views": len(ang),
                       "volume_zxy": a["dims"], "particles": n_part,
                       "order": "row walk (FP32 as its dependency levels), both precisions",
                       "slices_in_smem": bool(a["staged"])},
            "after_1_call": errors(1),
            "after_20_calls": errors(CALLS_PER_EQUIT),
            "fp32": {"wall_s": a["wall_s"], "icd_ms": a["icd_ms"], "calls": a["calls"],
                     "cost": a["cost"]},
            "fp64": {"wall_s": b["wall_s"], "icd_ms": b["icd_ms"], "calls": b["calls"],
                     "cost": b["cost"]},
            "data_generation_s": gen_s}
    print(json.dumps(line))


def run_batch(args):
    import torch
    import build as pkg_build
    pkg_build.build()
    import mbir
    torch.cuda.set_device(0)
    r = batch_measure(mbir, args.series, batch_threads=args.batch_threads)
    line = {"metric": "batched time-to-tolerance speed-up vs one-at-a-time GPU path",
            "value": r["speedup"], "unit": "x", "higher_is_better": True, "n_gpus": 1,
            "data": "synthetic",
            "config": {"workload": f"batch-{args.series}-uneven-haadf", "series": args.series,
                       "voxels_total": r["voxels_total"], "tolerance": r["tolerance"],
                       "max_outer": r["max_outer"]},
            "sequential": r["sequential"], "batched": r["batched"]}
    print(json.dumps(line))


def serve_measure(mbir, n, rate, seed=2, one_at_a_time=True):
    """Served stream: Poisson arrivals (mean `rate` requests/s) of mixed HAADF/BF requests from
    the uneven size distribution plus 5% of the 512x256x128 / 61-view shape, each to a 1e-4
    relative cost tolerance; p50/p99 latency and throughput with continuous batching, and
    (optionally) with the same requests served one at a time."""
    data = uneven_series(n, seed=seed, large_frac=0.05, bf_frac=0.3)
    rng = np.random.default_rng(seed + 1)
    gaps = rng.exponential(1.0 / rate, n)

    def submit_all(server):
        ids = []
        t0 = time.perf_counter()
        for item, gap in zip(data, gaps):
            mod, y, ang, th = item
            p = params_for(mbir, th, mod, outer=200)
            ids.append(server.submit(p, y, ang, max_outer=200 if mod == "BF" else 60, tol=1e-4))
            time.sleep(gap)
        for rid in ids:
            server.wait(rid, timeout=3600)
        return time.perf_counter() - t0

    with mbir.Server(0, 0, 0) as s:
        wall = submit_all(s)
        st = s.stats()
        served = {"wall_s": wall, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms,
                  "mean_ms": st.mean_ms, "completed": st.completed, "failed": st.failed,
                  "peak_active": st.peak_active, "requests_per_s": st.completed / wall,
                  "voxel_updates_per_s": st.voxel_updates / wall}
    out = {"requests": n, "arrival_rate_per_s": rate, "bf_fraction": 0.3,
           "large_fraction": 0.05, "tolerance": 1e-4, "continuous_batching": served}
    if one_at_a_time:
        with mbir.Server(0, 0, 1) as s:
            wall1 = submit_all(s)
            st = s.stats()
            out["one_at_a_time"] = {"wall_s": wall1, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms,
                                    "requests_per_s": st.completed / wall1}
        out["throughput_ratio"] = (served["requests_per_s"] /
                                   max(out["one_at_a_time"]["requests_per_s"], 1e-12))
    return out


def run_serve(args):
    import torch
    import build as pkg_build
    pkg_build.build()
    import mbir
    torch.cuda.set_device(0)
    r = serve_measure(mbir, args.series, args.rate)
    line = {"metric": "served p50/p99 request latency and throughput",
            "value": r["continuous_batching"]["p99_ms"], "unit": "ms (p99)",
            "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
            "config": {"workload": f"serve-poisson-{args.rate:g}rps", "requests": args.series,
                       "bf_fraction": 0.3, "large_fraction": 0.05, "tolerance": 1e-4},
            "continuous_batching": r["continuous_batching"],
            "one_at_a_time": r.get("one_at_a_time"), "throughput_ratio": r.get("throughput_ratio")}
    print(json.dumps(line))


def e2e_run(mbir, args, y, ang, th, mod, device):
    """One reconstruction through the C ABI from host buffers: create, upload, set-up and
    projection, the calls with offset and variance updates, read-back of the volume."""
    bf = mod == "BF"
    n_outer = CALLS_PER_EQUIT if bf else 3
    pe = params_for(mbir, th, mod, outer=n_outer, inner=1)
    pe.device = device
    if args.call_schedule is not None:
        pe.call_schedule = args.call_schedule
    if args.lane_shape is not None:
        pe.lane_shape = args.lane_shape
    t0 = time.perf_counter()
    with mbir.Engine(pe) as e2:
        e2.set_sinogram(y, ang)
        e2.run()
        host_vol = e2.volume()
        s2 = e2.status()
    dt = time.perf_counter() - t0
    return {"value": s2.voxels_updated / dt, "unit": "voxel-updates/s",
            "h2d_bytes_per_step": int(y.nbytes), "d2h_bytes_per_step": int(host_vol.nbytes),
            "step": f"mbir_create + mbir_set_sinogram + mbir_run ({n_outer} outer iterations: "
                    "call, offset and variance updates) + mbir_get_volume, host buffers",
            "wall_s": dt}


def e2e_cold(args, device):
    """e2e_run in a fresh Python process (nothing of this process's CUDA state is reused)."""
    cmd = [sys.executable, os.path.abspath(__file__), "--e2e-child", "--workload", args.workload,
           "--device", str(device)]
    if args.call_schedule is not None:
        cmd += ["--call-schedule", str(args.call_schedule)]
    if args.lane_shape is not None:
        cmd += ["--lane-shape", str(args.lane_shape)]
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
        return json.loads(r.stdout.strip().splitlines()[-1])
    except Exception:
        return None


def run_e2e_child(args):
    import build as pkg_build
    pkg_build.build()
    y, ang, th, mod = make_data(args.workload, seed=0)
    import mbir  # the library loads here, outside the timed region; the device context does not
    print(json.dumps(e2e_run(mbir, args, y, ang, th, mod, args.device)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    choices=sorted(WORKLOADS) + ["batch-64", "serve-poisson",
                                                 PRECISION_WORKLOAD])
    ap.add_argument("--series", type=int, default=64, help="batch/serve: number of requests")
    ap.add_argument("--rate", type=float, default=20.0, help="serve: mean arrivals per second")
    ap.add_argument("--no-batch", action="store_true",
                    help="default line: skip the batched time-to-tolerance measurement")
    ap.add_argument("--no-serve", action="store_true",
                    help="default line: skip the served-stream measurement")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--batch-threads", type=int, default=None,
                    help="CTA size of the persistent batched sweep (512 or 256)")
    ap.add_argument("--lane-shape", type=int, default=None,
                    help="voxel-group shape (1 16x4, 2 32x2, 3 32x3, 4 32x5; default autotuned)")
    ap.add_argument("--call-schedule", type=int, default=None,
                    help="BF NHICD call schedule (0 colour classes, 1 row walk, 2 levels)")
    ap.add_argument("--e2e-child", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--device", type=int, default=0, help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.e2e_child:
        run_e2e_child(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "batch-64":
        run_batch(args)
        return
    if args.workload == "serve-poisson":
        run_serve(args)
        return
    if args.workload == PRECISION_WORKLOAD:
        run_precision(args)
        return

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    import build as pkg_build
    pkg_build.build()
    import mbir

    y, ang, th, mod = make_data(args.workload, seed=rank)
    bf = mod == "BF"
    p = params_for(mbir, th, mod)
    p.device = local
    if args.call_schedule is not None:
        p.call_schedule = args.call_schedule
    if args.lane_shape is not None:
        p.lane_shape = args.lane_shape
    eng = mbir.Engine(p)
    eng.set_sinogram(y, ang)
    eng.prepare()
    nz, nx, ny = eng.dims()[:3]
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")
    calls_per_step = CALLS_PER_EQUIT if bf else 1
    ncall = [0]

    def step():
        tot = np.zeros(4)
        for _ in range(calls_per_step):
            k = ncall[0]
            tot += eng.sweep(0 if k == 0 else 1, 0)  # zero skipping after the first call
            ncall[0] += 1
        return tot

    for _ in range(args.warmup):
        step()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    per_ms = []
    upd = 0.0
    visited = 0.0
    barrier()
    st0 = eng.status()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))
            torch.cuda.synchronize()
            before = eng.status().icd_ms_total
            s = step()
            per_ms.append(eng.status().icd_ms_total - before)
            upd += s[3]
            visited += s[2] + s[3]
    barrier()
    st1 = eng.status()
    # the sweep kernels' own device time (events around the colour launches) and the host time
    # spent building level schedules, both inside the ICD interval above
    kernel_ms_step = (st1.kernel_ms_total - st0.kernel_ms_total) / args.steps
    sched_ms_step = (st1.sched_ms_total - st0.sched_ms_total) / args.steps
    colour_ms_step = (st1.colour_ms_total - st0.colour_ms_total) / args.steps
    total_ms = float(np.sum(per_ms))
    if dist is not None:
        t = torch.tensor([total_ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / args.steps
    value = world * upd / (total_ms / 1e3)
    st = eng.status()

    # roofline of the ICD kernels: algorithmic bytes per updated voxel = 8 F L + 8
    # (+ 5 F L for bright field: FP32 weight + u8 selector per footprint entry)
    f_mean = st.footprint_entries / float(nz * nx)
    per_vox = (13.0 if bf else 8.0) * f_mean * st.t_rows + 8.0
    bytes_step = (upd / args.steps) * per_vox
    peak, peak_kind = load_peaks()
    achieved = bytes_step / (kernel_ms_step / 1e3) / 1e9
    launches = calls_per_step * 3  # two colour launches + one stats reduction per call
    traffic = None
    tp = os.path.join(ROOT, "profiles", "icd_sweep_traffic.json")
    if os.path.exists(tp):
        try:
            with open(tp) as f:
                ent = json.load(f).get(args.workload)
            traffic = ent.get("bytes_per_launch") if isinstance(ent, dict) else ent
        except Exception:
            traffic = None

    cfg = workload_config(args.workload)
    assert cfg["volume_zxy"] == [nz, nx, ny], (cfg, (nz, nx, ny))
    out = {"metric": METRIC, "value": value, "unit": "voxel-updates/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic",
           "config": cfg,
           "details": {"order": "parallel (red/black y, conflict-free x)",
                      "replicas": world,
                      "voxels_updated_per_step": upd / args.steps,
                      "voxels_visited_per_step": visited / args.steps,
                      "slices_in_smem": bool(st.staged), "x_stride": st.stride,
                      "sweep_kernel_ms_per_step": kernel_ms_step,
                      "host_schedule_ms_per_step": sched_ms_step,
                      "colour_schedule_ms_per_step": colour_ms_step,
                      "levels_last_call": st.sched_levels},
           "gpu_launches": launches * args.steps,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "traffic": traffic,
                        "peak_source": peak_kind,
                        "algorithmic_bytes_per_step": bytes_step,
                        "algorithmic_bytes_per_launch": bytes_step / (2 * calls_per_step),
                        "traffic_unit": "bytes per colour launch (ncu capture)",
                        "bytes_model": ("13*F*L+8" if bf else "8*F*L+8") +
                                       " per updated voxel, F=A-column nnz, L=t rows",
                        "kernel": "sweep_kernel (two colour launches per call)",
                        "kernel_ms_per_launch": kernel_ms_step / (2 * calls_per_step)},
           "clocks": clk.summary()}

    if not args.no_e2e:
        # end to end through the C ABI from host buffers: cold, in a fresh process (CUDA context,
        # module load, set-up, autotuning all inside the timed region), and warm, in this
        # process after the timed engine (module loaded, shape tuning cached)
        warm = e2e_run(mbir, args, y, ang, th, mod, local)
        barrier()
        cold = e2e_cold(args, local)
        out["e2e"] = dict(cold) if cold else dict(warm)
        out["e2e"]["value"] *= world
        out["e2e"]["process"] = "fresh" if cold else "warm (fresh-process run failed)"
        out["e2e_warm"] = dict(warm, value=warm["value"] * world)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_reference_sample(args.workload)
    if rank == 0 and not args.no_batch:
        # the metric's second part: time to a 1e-4 relative cost tolerance, batched against the
        # plain one-reconstruction-at-a-time GPU path (16 uneven series; --workload batch-64
        # runs the full 64)
        out["time_to_converge"] = batch_measure(mbir, 16, batch_threads=args.batch_threads)
    if rank == 0 and not args.no_serve:
        # the third part: p50/p99 request latency of the served stream, at the benchmark's 20
        # requests/s (more than one GPU serves: the queue grows) and at 2 requests/s
        out["serving"] = {"rate_20": serve_measure(mbir, 24, 20.0, one_at_a_time=True),
                          "rate_2": serve_measure(mbir, 12, 2.0, one_at_a_time=False)}
    if rank == 0:
        print(json.dumps(out))
    eng.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
