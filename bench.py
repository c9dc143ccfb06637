#!/usr/bin/env python3
"""Throughput of brille's ir_interpolate_at query path on GB300.

One step = one ir_interpolate_at pass over one batch of seeded synthetic q
(uniform in [-L, L]³ r.l.u.) on the workload's trellis.  Default workload:
P6₃/mmc, a = 3.2 Å, c = 5.2 Å, 16 atoms (48 modes), 199 272-vertex trellis,
eigenvalues plus Γ-rotated eigenvectors at the reference's precision: FP64
vertex data, FP64 arithmetic, float64 / complex128 outputs, 1e7 q per step
in [-2, 2]³.  The outputs of one step (373 GB) exceed HBM, so each step
streams its q through one output buffer in chunks.

Reported (one JSON line from rank 0):
  value      q-points/s, all ranks, inputs and outputs resident in HBM
  e2e        the same 1e7 q per step through the public API with Q in pinned
             host memory and outputs copied into a pinned host buffer
             (host→device and device→host copies inside the timed region),
             beside the median of plain device→host copies sampled between
             the steps
  roofline   the dominant kernel's algorithmic bytes over its CUDA-event time
             against the measured HBM copy bandwidth (and, for the FP64
             gather, its FP64 instruction rate against the FP64 pipe)
  variants   FP32 and BF16 vertex storage (f32 / c64 outputs): throughput
             and error against the FP64 outputs on the same q
  cpu_baseline  the CPU oracle (a restatement of the reference's OpenMP
             path) on a bounded sample, on this host's cores

`--impl reference` times that CPU implementation alone (the reference's own
build needs HDF5 and generated headers that this toolchain lacks).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (crystal builder, node volume as a fraction of the zone, q half-range, q per step)
    "hex16": ("hexagonal16", 2.4e-7, 2.0, 10_000_000),
    "hex16-small": ("hexagonal16", 1e-5, 2.0, 1 << 20),
    # small trellis and batch with the group sizes of the full runs, for ncu
    "hex16-profile": ("hexagonal16", 1e-4, 2.0, 1 << 17),
    "diamond8": ("diamond_conventional", 1 / 5000, 1.0, 1 << 22),
    "diamond2": ("diamond_primitive", 1 / 5000, 1.0, 1 << 22),
}


METRIC = "interp q-pts/s on 1 GB300 (learned+coarse vs plain GPU) at <=1e-3 meV max err"

# dram__bytes_read.sum + dram__bytes_write.sum of the dominant kernel per q,
# keyed by (workload, stage, storage): from ncu captures named in `source`
PROFILED_TRAFFIC = {
    ("hex16", "gather_vectors", "f32"): dict(bytes_per_q=(12_696_951_552 + 184_570_256_896) / 1e7,
                                             source="ncu, one full-size warp_gather_kernel launch (1e7 q)"),
}

# FP64 thread instructions (DFMA + DMUL + DADD) per q of the FP64 vectors
# gather: a per-q part plus the once-per-group antiphase pass shared by the
# group's q, fitted to two ncu captures on the 882-vertex P6_3/mmc trellis
# (131072 q: 26.1 q per group, 6.572e9; 45000 q: 18.0 q per group, 2.293e9);
# the FP64 pipe issues `lanes_per_sm_cycle` of them per SM and cycle
PROFILED_FP64 = {
    ("hex16", "gather_vectors", "f64"): dict(
        per_q=48_305.0, per_group=47_900.0, lanes_per_sm_cycle=2,
        source="ncu on the 882-vertex P6_3/mmc trellis at 26.1 and 18.0 q per group "
               "(50 140 and 50 960 FP64 instructions per q; pipe 87 % and 78 % busy over the launch), "
               "fitted as per_q + per_group / (q per group)"),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def build_workload(name, gpu_build=True):
    from brille_gb300 import workloads as W
    from brille_gb300.bz import BrillouinZone
    from brille_gb300.trellis import TrellisBuild

    builder, fraction, qr, _ = WORKLOADS[name]
    lat, masses = getattr(W, builder)()
    bz = BrillouinZone(lat)
    t = time.time()
    tr = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * fraction)
    build_s = dict(host=round(time.time() - t, 2))
    log(f"[setup] trellis {tr.summary()} in {time.time() - t:.1f}s")
    # the same trellis built on the GPU (cut cells fanned into tetrahedra
    # there): set-up time only, the query runs on the host-built tables
    try:
        if not gpu_build:
            raise RuntimeError("not built in this run")
        t = time.time()
        trg = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * fraction, backend="gpu")
        build_s["gpu"] = round(time.time() - t, 2)
        build_s["gpu_same_vertices"] = len(trg.vertices) == len(tr.vertices)
        log(f"[setup] trellis on the GPU {trg.summary()} in {build_s['gpu']:.1f}s")
        del trg
    except Exception as e:  # no GPU in this process: set-up timing only
        build_s["gpu"] = f"unavailable: {e}"
    model = W.bvk_for(lat, masses)
    qv = tr.vertices @ np.linalg.inv(lat.B)
    t = time.time()
    procs = min(16, os.cpu_count() or 1)
    w, v = model.modes(qv, chunk=2048, processes=procs if len(qv) > 8192 else 0)
    log(f"[setup] BvK modes for {len(qv)} vertices in {time.time() - t:.1f}s ({procs} processes)")
    return dict(name=name, lat=lat, bz=bz, tr=tr, model=model, w=w, v=v, q_range=qr, build_s=build_s)


def matched_plain(curve, rec, key):
    """The coarsest plain trellis of `curve` whose error `key` is at or
    below the record's, or None."""
    ok = [c for c in curve if c[key] <= rec[key]]
    return min(ok, key=lambda c: c["vertices"]) if ok else None


def bytes_per_q(B, n_atoms, out_f32):
    s = 4 if out_f32 else 8
    vals = B * s
    vecs = B * 3 * n_atoms * 2 * s
    return 24, vals, vecs


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.path = tempfile.mktemp(suffix=".csv")
        self.index = index
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            if len(r) < 9:
                continue
            for k, n in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


def cpu_baseline(wl, target_s=12.0, threads=0):
    """The oracle (CPU restatement of the reference's path) on a bounded sample."""
    from brille_gb300.tables import geometry_tables
    from oracle.oracle import Oracle

    t = geometry_tables(wl["bz"], wl["tr"])
    o = Oracle(t)
    w, v = wl["w"], wl["v"]
    nv, B = w.shape
    vals = (np.ascontiguousarray(w[:, :, None]), [1, 0, 0], 0, 3)
    vecs = (np.ascontiguousarray(v.reshape(nv, B, -1)), [0, 3 * v.shape[2], 0], 2, 1)
    rng = np.random.default_rng(123)
    qr = wl["q_range"]
    n = 256
    while True:
        Q = rng.uniform(-qr, qr, size=(n, 3))
        t0 = time.perf_counter()
        o.interpolate_at(Q, vals, vecs, threads=threads)
        dt = time.perf_counter() - t0
        if dt > target_s / 4 or n >= 1 << 22:
            break
        n = int(n * min(16, max(2, (target_s / 4) / max(dt, 1e-3))))
    n_final = max(n, int(n * target_s / max(dt, 1e-6)))
    Q = rng.uniform(-qr, qr, size=(n_final, 3))
    t0 = time.perf_counter()
    _, _, rc, _ = o.interpolate_at(Q, vals, vecs, threads=threads)
    dt = time.perf_counter() - t0
    cores = threads if threads > 0 else Oracle.max_threads()
    return dict(value=n_final / dt, unit="q-points/s", cores=cores, kind="port",
                sample=f"{n_final} q uniform in [-{qr},{qr}]^3 on the same trellis, FP64, values+vectors, "
                       f"serial move stage and OpenMP locate/gather/rotate as the reference", seconds=dt, rc=rc)


def run_reference(args, rank):
    if rank != 0:
        return
    wl = build_workload(args.workload, gpu_build=False)
    vals = []
    import oracle.oracle as orc
    nthreads = orc.Oracle.max_threads()
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(wl, target_s=max(2.0, 60.0 / (args.steps + args.warmup)), threads=nthreads)
        if i >= args.warmup:
            vals.append(r)
    value = float(np.median([r["value"] for r in vals]))
    out = dict(metric=METRIC,
               impl="reference", value=value, unit="q-points/s", n_gpus=0, steps=args.steps, warmup=args.warmup,
               ms_per_step=float(np.median([r["seconds"] for r in vals])) * 1e3, higher_is_better=True,
               scaling="weak", vs_baseline=None, dtype="f64", data="synthetic (seeded BvK model, uniform q)",
               config=dict(workload=args.workload, trellis_vertices=int(len(wl["tr"].vertices)),
                           modes=int(wl["w"].shape[1])),
               cpu_baseline=dict(value=value, unit="q-points/s", cores=vals[-1]["cores"], kind="port",
                                 sample=vals[-1]["sample"]),
               e2e=dict(value=value, unit="q-points/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(out), flush=True)


def run_precision(args):
    """FP32 and BF16-eigenvector storage against the FP64 path (which equals
    the oracle: bit-exact eigenvalues, eigenvectors within 1e-12) on
    n q, half uniform in [-L, L]³ and half within 1e-6 r.l.u. of trellis
    faces, knot planes and high-symmetry lines; plus the FP64 path against the
    exact BvK model on a subsample."""
    import torch

    from brille_gb300 import BZTrellisQdc
    from brille_gb300 import workloads as W

    wl = build_workload(args.workload)
    B, na = wl["w"].shape[1], wl["v"].shape[2]
    n = args.q_per_step or 10_000_000
    half = n // 2
    rng = np.random.default_rng(5)
    Q = np.concatenate([rng.uniform(-wl["q_range"], wl["q_range"], size=(half, 3)),
                        W.near_boundary_q(wl["bz"], wl["tr"], n - half, seed=6)])
    grids = {}
    for st in ("f64", "f32", "bf16"):
        g = BZTrellisQdc(wl["bz"], trellis=wl["tr"])
        g.fill(wl["w"], [1, 0, 0, 0, 3], wl["v"], [0, 3 * na, 0, 2, 1], storage=st)
        grids[st] = g
    dev = torch.device("cuda")
    # chunks of at most ~4 GB of complex128 eigenvectors per storage
    chunk = int(max(4096, min(1 << 20, (4 << 30) // (B * na * 3 * 16))))
    acc = {st: dict(vmax=0.0, vsq=0.0, omax=0.0, osum=0.0, cnt=0, gmax=0.0, gsum=0.0, nbad=0)
           for st in ("f32", "bf16")}
    degen_tol = 1e-3  # meV: modes closer than this form one degenerate group
    for a in range(0, n, chunk):
        b_ = min(n, a + chunk)
        m = b_ - a
        Qd = torch.from_numpy(Q[a:b_]).to(dev)
        out = {}
        for st, g in grids.items():
            v = torch.empty((m, B), dtype=torch.float64, device=dev)
            c = torch.empty((m, B, na, 3), dtype=torch.complex128, device=dev)
            g.query_into(Qd, m, v, c)
            out[st] = (v, c)
        v64, c64 = out["f64"]
        for st in ("f32", "bf16"):
            v, c = out[st]
            dv = (v - v64).abs()
            acc[st]["vmax"] = max(acc[st]["vmax"], float(dv.max()))
            acc[st]["vsq"] += float((dv ** 2).sum())
            ov = (torch.conj(c64) * c).sum(dim=(2, 3)).abs() / (
                torch.linalg.vector_norm(c64, dim=(2, 3)) * torch.linalg.vector_norm(c, dim=(2, 3))).clamp_min(1e-300)
            e = 1 - ov
            acc[st]["omax"] = max(acc[st]["omax"], float(e.max()))
            acc[st]["osum"] += float(e.sum())
            acc[st]["cnt"] += e.numel()
            # degenerate-subspace overlap: 1 − sqrt(Σ_{j in G(b)} |<v̂_ref_b, v̂_j>|²)
            # over the group G(b) of modes within degen_tol of each other (FP64 eigenvalues)
            gid = torch.cat([torch.zeros((m, 1), dtype=torch.int64, device=dev),
                             torch.cumsum((v64[:, 1:] - v64[:, :-1]).abs() >= degen_tol, dim=1)], dim=1)
            r = c64 / torch.linalg.vector_norm(c64, dim=(2, 3), keepdim=True).clamp_min(1e-300)
            u = c / torch.linalg.vector_norm(c, dim=(2, 3), keepdim=True).clamp_min(1e-300)
            tot = torch.zeros((m, B), dtype=torch.float64, device=dev)
            # groups are runs of consecutive modes: stop at the first distance
            # with no pair inside one group
            for d in range(B):
                same = gid[:, :B - d] == gid[:, d:]
                if not bool(same.any()):
                    break
                for a0, b0 in ((0, d), (d, 0)) if d else ((0, 0),):
                    o = (torch.conj(r[:, a0:a0 + B - d]) * u[:, b0:b0 + B - d]).sum(dim=(2, 3)).abs() ** 2
                    tot[:, a0:a0 + B - d] += torch.where(same, o, torch.zeros_like(o))
            ge = 1 - torch.sqrt(tot)
            acc[st]["gmax"] = max(acc[st]["gmax"], float(ge.max()))
            acc[st]["gsum"] += float(ge.sum())
            acc[st]["nbad"] += int((ge > 1e-3).sum())
    res = {}
    for st, a_ in acc.items():
        res[st] = dict(eig_max_abs_meV=a_["vmax"], eig_rms_meV=(a_["vsq"] / (n * B)) ** 0.5,
                       overlap_loss_max=a_["omax"], overlap_loss_mean=a_["osum"] / max(a_["cnt"], 1),
                       subspace_overlap_loss_max=a_["gmax"],
                       subspace_overlap_loss_mean=a_["gsum"] / max(a_["cnt"], 1),
                       subspace_overlap_loss_above_0p001_fraction=a_["nbad"] / max(a_["cnt"], 1),
                       degenerate_group_tol_meV=degen_tol)
    # the FP64 path against the exact model (interpolation error of the trellis itself)
    ns = 200_000
    Qs = Q[rng.integers(0, n, ns)]
    gv, _ = grids["f64"].ir_interpolate_at(Qs)
    ex, _ = wl["model"].modes(Qs, chunk=8192, processes=min(16, os.cpu_count() or 1))
    err = np.abs(gv - ex)
    res["f64_vs_exact_bvk"] = dict(sample=ns, eig_max_abs_meV=float(err.max()),
                                   eig_rms_meV=float(np.sqrt((err ** 2).mean())),
                                   eig_p99_meV=float(np.quantile(err, 0.99)))
    out = dict(mode="precision", workload=args.workload, q=n,
               q_set="half uniform in [-%g,%g]^3, half within 1e-6 r.l.u. of tetrahedron faces, knot planes "
                     "and high-symmetry lines (random symmetry images and zones)" % (wl["q_range"], wl["q_range"]),
               reference="FP64 path (equal to the CPU oracle: bit-exact eigenvalues, eigenvectors within 1e-12)",
               trellis_vertices=int(len(wl["tr"].vertices)), modes=int(B), results=res)
    print(json.dumps(out), flush=True)


BATCH_GROUPS = ("P-1", "P2/m", "Pmmm", "P4/mmm", "R-3m", "P6/mmm", "Fm-3m", "Im-3m")


def _batch_item(k, seed, vmin, vmax):
    """One interpolator of the batched workload, built in a worker process:
    space group k mod 8, seeded lattice (3-8 Å, free angles 60-120°), 1-6
    symmetric orbits (≤ 32 atoms), trellis aimed at a vertex count
    log-uniform in [vmin, vmax]."""
    from scipy.spatial import ConvexHull

    from brille_gb300 import workloads as W
    from brille_gb300.bz import BrillouinZone
    from brille_gb300.trellis import TrellisBuild

    rng = np.random.default_rng(seed)
    name = BATCH_GROUPS[k % len(BATCH_GROUPS)]
    lat, masses = W.random_crystal(name, int(rng.integers(1, 7)), seed=seed, max_atoms=32)
    bz = BrillouinZone(lat)
    target = float(np.exp(rng.uniform(np.log(vmin), np.log(vmax))))
    ratio = bz.volume / ConvexHull(bz.ir_vertices_invA).volume
    frac = 4.0 / (ratio * target)
    tr = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * frac)
    # one correction: vertex count scales about as 1/node volume
    if not 0.67 < len(tr.vertices) / target < 1.5:
        tr = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * frac * len(tr.vertices) / target)
    return name, lat, masses, tr


def run_batch(args):
    """64 interpolators of different space groups, trellises and mode counts,
    ragged q counts (log-uniform 1e3-5e6, 5e7 in all), values + Γ-rotated
    eigenvectors in FP32 from each crystal's Born-von Karman model, answered
    by the batched path: one persistent launch per stage, autotuned, replayed
    from a captured CUDA graph.  All outputs of 5e7 q do not fit in HBM, so
    the q run in W waves of one graph replay each into reused output
    buffers."""
    import torch

    from brille_gb300 import BZTrellisQdc
    from brille_gb300.batch import BatchQuery
    from brille_gb300.bvk import spawn_pool
    from brille_gb300.bz import BrillouinZone

    n_items = args.batch_items
    total_q = args.q_per_step or 50_000_000
    vmin, vmax = 2e3, args.batch_vmax
    t0 = time.time()
    procs = min(16, os.cpu_count() or 1)
    with spawn_pool(procs) as ex:
        items = list(ex.map(_batch_item, range(n_items), [9000 + k for k in range(n_items)], [vmin] * n_items,
                            [vmax] * n_items))
    log(f"[batch] {n_items} trellises in {time.time() - t0:.1f}s")
    dev = torch.device("cuda")
    gen = torch.Generator(device=dev)
    gen.manual_seed(77)
    from brille_gb300 import workloads as W
    from brille_gb300.bvk import modes_each

    grids, B, na, V = [None] * len(items), [0] * len(items), [0] * len(items), [0] * len(items)

    # vertex data from each crystal's BvK model, one item at a time through
    # one process pool; each item's data go to its handle (FP32 on the
    # device) before the next item's are formed
    def fill(i, w, v):
        name, lat, masses, tr = items[i]
        nat = len(lat.basis.positions)
        g = BZTrellisQdc(BrillouinZone(lat), trellis=tr)
        g.fill(torch.from_numpy(w).to(dev, torch.float32), [1, 0, 0, 0, 3],
               torch.from_numpy(v).to(dev, torch.complex64), [0, 3 * nat, 0, 2, 1], storage="f32")
        g._fill["values"] = g._fill["vectors"] = None  # the device copy is the handle's
        grids[i], B[i], na[i], V[i] = g, 3 * nat, nat, len(tr.vertices)
        if i % 16 == 15:
            log(f"[batch] BvK data of {i + 1} items in {time.time() - t0:.1f}s")

    modes_each([(W.bvk_for(lat, masses), tr.vertices @ np.linalg.inv(lat.B)) for _, lat, masses, tr in items], fill,
               processes=procs)
    torch.cuda.empty_cache()
    log(f"[batch] filled in {time.time() - t0:.1f}s; vertices {min(V)}-{max(V)}, modes {min(B)}-{max(B)}")
    # ragged q counts: log-uniform in [1e3, 5e6], scaled to the total
    rng = np.random.default_rng(5)
    nq = np.exp(rng.uniform(np.log(1e3), np.log(5e6), n_items))
    for _ in range(20):
        nq = np.clip(nq * total_q / nq.sum(), 1e3, 5e6)
    nq = np.maximum(1, np.round(nq)).astype(np.int64)
    per_q = np.array([b * 4 + b * 3 * a * 8 for b, a in zip(B, na)], dtype=np.float64)  # f32 / c64 outputs
    free, _ = torch.cuda.mem_get_info()
    budget = 0.55 * free - n_items * (1 << 20)
    waves = max(1, int(np.ceil(float((nq * (per_q + 24 + 200)).sum()) / budget)))
    m = [int((n + waves - 1) // waves) for n in nq]
    done_q = waves * sum(m)
    log(f"[batch] {int(nq.sum())} q in {waves} waves of {sum(m)} q; outputs {float((per_q * m).sum()) / 1e9:.1f} GB "
        f"per wave")
    Qall = [(torch.rand((waves * mi, 3), generator=gen, device=dev, dtype=torch.float64) * 2 - 1) for mi in m]
    bq = BatchQuery(grids, m, out_f32=True)
    vals, vecs = bq.outputs()
    stream = torch.cuda.Stream(dev)
    sp = stream.cuda_stream

    def wave_io(w):
        bq.set_io([q[w * mi:(w + 1) * mi] for q, mi in zip(Qall, m)], vals, vecs)

    wave_io(0)
    t = time.time()
    cfg = bq.tune(sp, reps=2)
    log(f"[batch] tuned in {time.time() - t:.1f}s: {cfg}")
    bq.capture(sp)
    for w in range(min(args.warmup, waves)):
        wave_io(w)
        bq.launch(sp)
        bq.sync(sp)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = bq.launch_count()
    # per wave: events around each replay, so that the host's set_io and
    # synchronisation between replays (the bubble) is measured apart
    wev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(waves)]
    with Clocks(0) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for w in range(waves):
            wave_io(w)
            wev[w][0].record(stream)
            bq.launch(sp)
            wev[w][1].record(stream)
            bq.sync(sp)  # the next set_io rewrites the pinned tables this replay reads
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    replay_ms = [a.elapsed_time(b) for a, b in wev]
    launches = bq.launch_count() - l0
    # the same waves, one query per grid
    for i, g in enumerate(grids):
        if m[i]:
            g.query_into(Qall[i][:m[i]], m[i], vals[i], vecs[i], out_f32=True, stream=sp)
    torch.cuda.synchronize()
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # per item: events around its query in the first wave
    iev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in grids]
    ev2.record(stream)
    for w in range(waves):
        for i, g in enumerate(grids):
            if m[i]:
                if w == 0:
                    iev[i][0].record(stream)
                g.query_into(Qall[i][w * m[i]:(w + 1) * m[i]], m[i], vals[i], vecs[i], out_f32=True, async_=True,
                             stream=sp)
                if w == 0:
                    iev[i][1].record(stream)
    ev3.record(stream)
    for g in grids:
        g.sync(sp)
    torch.cuda.synchronize()
    ms_single = ev2.elapsed_time(ev3)
    items_ms = [iev[i][0].elapsed_time(iev[i][1]) if m[i] else 0.0 for i in range(len(grids))]
    order = np.argsort(items_ms)[::-1]
    per_item = [dict(item=int(i), group=items[i][0], atoms=int(na[i]), modes=int(B[i]), vertices=int(V[i]),
                     q=int(m[i]), ms=round(items_ms[i], 3),
                     gbs=round(float(per_q[i]) * m[i] / max(items_ms[i], 1e-9) / 1e6, 1)) for i in order[:12]]
    log(f"[batch] per item, first wave, slowest first: {per_item}")
    out_bytes = float((per_q * m).sum()) * waves
    peaks = measured_peaks()
    peak = float(peaks["hbm_gbs"]) if peaks else 6800.0
    achieved = out_bytes / (ms / 1e3) / 1e9
    out = dict(mode="batch", metric="interp q-pts/s, 64 interpolators batched", value=done_q / (ms / 1e3),
               unit="q-points/s", ms_total=ms, waves=waves, q_total=done_q, n_items=n_items,
               per_grid_queries=dict(value=done_q / (ms_single / 1e3), ms_total=ms_single,
                                     note="the same waves as one ir_interpolate_at call per grid, queued async"),
               speedup_vs_per_grid=ms_single / ms,
               per_grid_first_wave_ms=round(float(sum(items_ms)), 2), slowest_items_first_wave=per_item,
               replay_ms=[round(x, 2) for x in replay_ms],
               between_replays_ms=round(ms - sum(replay_ms), 2),
               config=dict(space_groups=list(BATCH_GROUPS), vertices=[int(min(V)), int(max(V)), int(np.median(V))],
                           modes=[int(min(B)), int(max(B))], atoms=[int(min(na)), int(max(na))],
                           q_per_item=[int(nq.min()), int(nq.max())], q_range=1.0, storage="f32",
                           outputs="f32 values + c64 Gamma-rotated eigenvectors",
                           data="synthetic: each crystal's seeded BvK model at its trellis vertices",
                           tuned=cfg, graph="captured once, replayed per wave with new Q pointers"),
               roofline=dict(bound="hbm", kernel="whole batch (outputs only)", achieved=round(achieved, 1),
                             peak=peak, unit="GB/s", frac=round(achieved / peak, 4),
                             algorithmic_bytes=out_bytes, traffic=None),
               gpu_launches=int(launches), clocks=clk.summary())
    print(json.dumps(out), flush=True)


# plain trellises of the learned comparison (fractions of the zone volume)
# and the coarse trellises the learned residual corrects
LEARNED_PLAIN = (("bz/200", 1 / 200), ("bz/625", 1 / 625), ("bz/5000", 1 / 5000), ("bz/40000", 1 / 40000),
                 ("bz/320000", 1 / 320000), ("bz/2560000", 1 / 2560000))
LEARNED_COARSE = (("bz/625", 1 / 625), ("bz/200", 1 / 200))


def run_sqw(args):
    """The structure factor of the interpolated modes (the consumer brille
    feeds) on the headline workload: values + S per q and mode from the
    fused gather, against values + eigenvectors from ir_interpolate_at on
    the same q, both with Q and outputs in HBM."""
    import torch

    from brille_gb300 import BZTrellisQdc

    wl = build_workload(args.workload)
    B, na = wl["w"].shape[1], wl["v"].shape[2]
    grid = BZTrellisQdc(wl["bz"], trellis=wl["tr"])
    grid.fill(wl["w"], [1, 0, 0, 0, 3], wl["v"], [0, 3 * na, 0, 2, 1], storage=args.storage)
    rng = np.random.default_rng(5)
    grid.set_atoms(rng.uniform(0.3, 1.0, na), np.asarray(wl["lat"].basis.positions, float))
    n = args.q_per_step or WORKLOADS[args.workload][3]
    dev = torch.device("cuda")
    gen = torch.Generator(device=dev)
    gen.manual_seed(1000)
    Q = (torch.rand((n, 3), generator=gen, device=dev, dtype=torch.float64) * 2 - 1) * wl["q_range"]
    vals = torch.empty((n, B), dtype=torch.float32, device=dev)
    sf = torch.empty((n, B), dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)
    sp = stream.cuda_stream
    if args.tuning:
        grid.set_tuning([int(x) for x in args.tuning.split(",")])
    elif not args.no_tune:
        grid.tune(Q, out_f32=True, reps=2, stream=sp, values_out=vals,
                  vectors_out=torch.empty((n, B, na, 3), dtype=torch.complex64, device=dev))
        torch.cuda.empty_cache()

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        grid.sync(sp)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        grid.profile(True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        grid.sync(sp)
        torch.cuda.synchronize()
        stage_ms = grid.stage_times()[0]
        grid.profile(False)
        return e0.elapsed_time(e1) / args.steps, [round(x / args.steps, 3) for x in stage_ms]

    ms_sf, st_sf = timed(lambda: grid.structure_factor_into(Q, n, vals, sf, async_=True, stream=sp))
    vecs = torch.empty((n, B, na, 3), dtype=torch.complex64, device=dev)
    ms_v, st_v = timed(lambda: grid.query_into(Q, n, vals, vecs, out_f32=True, async_=True, stream=sp))
    out = dict(mode="sqw", metric="q-points/s, values + structure factor per mode", value=n / (ms_sf / 1e3),
               unit="q-points/s", ms_per_step=ms_sf, steps=args.steps, warmup=args.warmup,
               stage_ms_per_step=dict(zip(["locate", "grouping", "values", "structure_factor"], st_sf)),
               vectors_path=dict(value=n / (ms_v / 1e3), ms_per_step=ms_v,
                                 stage_ms_per_step=dict(zip(["locate", "grouping", "values", "vectors"], st_v)),
                                 note="the same q through ir_interpolate_at, eigenvectors written to HBM"),
               speedup_vs_vectors=ms_v / ms_sf,
               config=dict(workload=args.workload, q_per_step=n, modes=B, atoms=na, storage=args.storage,
                           outputs="f32 values + f32 S per mode (8 B per q and mode) vs c64 eigenvectors "
                                   f"({24 * na} B per q and mode)"),
               data="synthetic (seeded BvK model, random atom weights), q uniform")
    print(json.dumps(out), flush=True)


def run_sort(args):
    """sort() on the headline workload: the mode permutation of every vertex
    pair that shares a node (brx_sort, FP64 costs on FP64 storage, exact
    assignment), against the CPU oracle of the same computation on a bounded
    sample of pairs on this host's cores."""
    import torch

    from brille_gb300 import BZTrellisQdc
    from oracle import oracle as O

    wl = build_workload(args.workload)
    B, na = wl["w"].shape[1], wl["v"].shape[2]
    grid = BZTrellisQdc(wl["bz"], trellis=wl["tr"])
    grid.fill(wl["w"], [1, 0, 0, 0, 3], wl["v"], [0, 3 * na, 0, 2, 1], storage="f64")
    t = time.time()
    keys = grid.permutation_keys()
    log(f"[setup] {keys.size} permutation keys in {time.time() - t:.1f}s")
    pairs = keys.size // 2
    stream = torch.cuda.Stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dev_ms, wall_ms = [], []
    for rep in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        e0.record(stream)
        grid.sort(stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        if rep >= args.warmup:
            wall_ms.append((time.perf_counter() - t) * 1e3)
            dev_ms.append(e0.elapsed_time(e1))
    k, perms = grid.permutation_table()
    moved = int((perms != np.arange(B)).any(axis=1).sum())
    ms = float(np.median(dev_ms))
    # FP64 flops of the Hermitian products alone: B² pairs × s elements × 8
    span = 3 * na
    flops = pairs * B * B * span * 8.0
    # CPU oracle on a bounded sample of pairs (both directions of each)
    nv = len(wl["tr"].vertices)
    i, j = keys // nv, keys % nv
    fwd = np.nonzero(i < j)[0]
    rng = np.random.default_rng(0)
    take = np.sort(rng.choice(fwd, size=min(len(fwd), 4000), replace=False))
    sample = np.unique(np.concatenate([keys[take], j[take] * nv + i[take]]))
    vals = (np.ascontiguousarray(wl["w"][:, :, None]), (1, 0, 0), 0, (1, 1, 1))
    vecs = (np.ascontiguousarray(wl["v"].reshape(nv, B, -1)), (0, span, 0), 0, (1, 1, 1))
    threads = os.cpu_count() or 1
    t = time.perf_counter()
    ref = O.sort_permutations(vals, vecs, sample, threads=threads)
    cpu_s = time.perf_counter() - t
    pos = np.searchsorted(k, sample)
    agree = float((perms[pos] == ref).all(axis=1).mean())
    out = dict(mode="sort", metric="vertex pairs sorted per second", value=pairs / (ms / 1e3), unit="pairs/s",
               ms_per_sort=ms, wall_ms_per_sort=float(np.median(wall_ms)), steps=args.steps, warmup=args.warmup,
               pairs=int(pairs), keys=int(keys.size), non_identity_keys=moved,
               fp64_hermitian_gflops=flops / (ms / 1e3) / 1e9,
               cpu_baseline=dict(value=len(take) / cpu_s, unit="pairs/s", cores=threads, kind="port",
                                 sample=f"{len(take)} random pairs of the same trellis (both keys each)"),
               oracle_agreement=agree,
               config=dict(workload=args.workload, modes=B, atoms=na, vertices=nv, storage="f64",
                           costs="|Δω| + sin² of the Hermitian angle (the reference's defaults)"),
               data="synthetic (seeded BvK model)")
    print(json.dumps(out), flush=True)


def learned_curve(args, n_eval, steps, warmup, plain=LEARNED_PLAIN, coarse=LEARNED_COARSE, log_progress=True):
    """The metric: learned residual on coarse trellises against plain
    trellises of increasing density, on the 2-atom FCC crystal (a = 4.96 Å,
    28 amu; BZ/5000 is the small plain configuration): max / RMS eigenvalue
    error against the exact FP64 BvK model on held-out uniform q in [-1,1]³,
    and eigenvalue throughput of each path on device-resident q.  The ratio
    is taken at matched accuracy: learned q/s over the q/s of the coarsest
    plain trellis whose max error is at or below the learned one."""
    import torch

    from brille_gb300 import workloads as W
    from brille_gb300.bz import BrillouinZone
    from brille_gb300.grid import BZTrellisQdd
    from brille_gb300.learned import ResidualModel
    from brille_gb300.trellis import TrellisBuild

    lat, masses = W.diamond_primitive()
    bz = BrillouinZone(lat)
    model = W.bvk_for(lat, masses)
    B = model.n_modes
    procs = min(16, os.cpu_count() or 1)
    Binv = np.linalg.inv(lat.B)
    dev = torch.device("cuda")
    n_train = args.train_q or 1_000_000
    t = time.time()
    Qt = np.random.default_rng(11).uniform(-1, 1, (n_train, 3))
    wt = model.frequencies(Qt, processes=procs)
    Qe = np.random.default_rng(12).uniform(-1, 1, (n_eval, 3))
    we = model.frequencies(Qe, processes=procs)
    if log_progress:
        log(f"[learned] exact BvK for {n_train} + {n_eval} q in {time.time() - t:.1f}s ({procs} processes)")
    Qd = torch.from_numpy(Qe).to(dev)
    Wd = torch.from_numpy(we).to(dev)
    out = torch.empty((n_eval, B), dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)
    sp = stream.cuda_stream

    def grid_at(frac):
        t0 = time.time()
        tr = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * frac)
        g = BZTrellisQdd(bz, trellis=tr)
        g.fill(model.frequencies(tr.vertices @ Binv, processes=procs if len(tr.vertices) > 20000 else 0)[:, :, None],
               [1, 0, 0, 0, 3], storage="f32")
        return g, time.time() - t0

    def errors(g):
        g.query_into(Qd, n_eval, out, None, out_f32=True, stream=sp)
        torch.cuda.synchronize()
        e = (out.double() - Wd).abs().flatten()
        return dict(max_meV=float(e.max()), rms_meV=float(e.square().mean().sqrt()),
                    p99_meV=float(torch.quantile(e[:1 << 24].float(), 0.99)),
                    p9999_meV=float(torch.quantile(e[:1 << 24].float(), 0.9999)))

    def throughput(g):
        for _ in range(warmup):
            g.query_into(Qd, n_eval, out, None, out_f32=True, async_=True, stream=sp)
            g.sync(sp)
        torch.cuda.synchronize()
        g.profile(True)
        l0 = g.launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            g.query_into(Qd, n_eval, out, None, out_f32=True, async_=True, stream=sp)
        ev1.record(stream)
        g.sync(sp)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / steps
        st_ms, _, _ = g.stage_times()
        g.profile(False)
        return dict(q_per_s=n_eval / (ms / 1e3), ms_per_step=ms, gpu_launches=int(g.launch_count() - l0),
                    stage_ms_per_step=dict(zip(["locate", "grouping", "values", "vectors"],
                                               [round(x / steps, 3) for x in st_ms])))

    curve = []
    for name, frac in plain:
        g, build_s = grid_at(frac)
        r = dict(trellis=name, vertices=int(len(g.trellis.vertices)), build_s=round(build_s, 1), **errors(g),
                 **throughput(g))
        curve.append(r)
        if log_progress:
            log(f"[learned] plain {name} ({r['vertices']} vertices): max {r['max_meV']:.3g} rms {r['rms_meV']:.3g} meV, "
                f"{r['q_per_s']:.3g} q/s")
        del g
    peaks = measured_peaks()
    learned = []
    for name, frac in coarse:
        g, _ = grid_at(frac)
        m = ResidualModel(B, seed=0)
        torch.cuda.synchronize()
        t0 = time.time()
        hist = m.train_on(g, Qt, wt, epochs=args.epochs, batch=4096, lr=2e-3, log=log if log_progress else None)
        torch.cuda.synchronize()
        r = dict(trellis=name, vertices=int(len(g.trellis.vertices)),
                 train=dict(samples=n_train, epochs=args.epochs, batch=4096, seconds=round(time.time() - t0, 2),
                            loss_first=hist[0], loss_last=hist[-1], params=m.n_params, d_in=m.d_in))
        plain_speed = throughput(g)
        m.attach(g)
        r.update(errors(g))
        r.update(throughput(g))
        mlp_ms = r["stage_ms_per_step"]["values"] - plain_speed["stage_ms_per_step"]["values"]
        flops_q = 2 * (m.d_in * 128 + 2 * 128 * 128 + 128 * m.n_out)
        if mlp_ms > 0:
            ach = flops_q * n_eval / (mlp_ms / 1e3) / 1e12
            pk = float(peaks["bf16_tflops"]) if peaks else 1900.0
            r["mlp_roofline"] = dict(bound="tensor", achieved=round(ach, 2), peak=pk, unit="TFLOP/s",
                                     frac=round(ach / pk, 4), flops_per_q=flops_q, ms_per_step=round(mlp_ms, 3),
                                     peak_source="measured" if peaks else "fallback")
        # matched accuracy: the coarsest plain trellis at or below this max error
        match = matched_plain(curve, r, "max_meV")
        if match:
            r["matched_plain"] = dict(trellis=match["trellis"], vertices=match["vertices"], max_meV=match["max_meV"],
                                      q_per_s=match["q_per_s"])
            r["ratio_at_matched_max_error"] = r["q_per_s"] / match["q_per_s"]
        else:
            finest = max(curve, key=lambda c: c["vertices"])
            r["matched_plain"] = None
            r["ratio_vs_finest_plain"] = r["q_per_s"] / finest["q_per_s"]
        # the same at matched RMS error (secondary; the metric is max error)
        mr = matched_plain(curve, r, "rms_meV")
        if mr:
            r["matched_plain_rms"] = dict(trellis=mr["trellis"], vertices=mr["vertices"], rms_meV=mr["rms_meV"],
                                          q_per_s=mr["q_per_s"])
            r["ratio_at_matched_rms_error"] = r["q_per_s"] / mr["q_per_s"]
        learned.append(r)
        if log_progress:
            log(f"[learned] learned {name}: max {r['max_meV']:.3g} rms {r['rms_meV']:.3g} meV, {r['q_per_s']:.3g} q/s")
        del g
    # plain max error against vertex count, fitted in log-log over the three
    # finest trellises (linear interpolation errs ~h near the Γ cone)
    fit = sorted(curve, key=lambda c: c["vertices"])[-3:]
    slope, icpt = np.polyfit(np.log([c["vertices"] for c in fit]), np.log([c["max_meV"] for c in fit]), 1)
    need = float(np.exp((np.log(1e-3) - icpt) / slope)) if slope < 0 else None
    return dict(crystal="FCC Fd-3m a=4.96 A, 2-atom primitive basis, 28 amu, 6 modes", q_eval=n_eval,
                q_eval_set="uniform in [-1,1]^3 r.l.u., seed 12 (held out)",
                train_set=f"{n_train} q uniform in [-1,1]^3 r.l.u., seed 11, folded into the wedge by the locate",
                exact="BvK eigenvalues (FP64 eigvalsh) at each q", outputs="f32 eigenvalues, storage f32",
                target="<=1e-3 meV max error", target_met=any(c["max_meV"] <= 1e-3 for c in curve + learned),
                plain_curve=curve, learned=learned,
                plain_max_error_fit=dict(slope_vs_vertices=float(slope),
                                         vertices_for_1e_3_meV=need))


def run_learned(args):
    """--mode learned: the full comparison on 1e7 held-out q."""
    res = learned_curve(args, args.q_per_step or 10_000_000, args.steps, args.warmup)
    print(json.dumps(dict(mode="learned", steps=args.steps, warmup=args.warmup, **res)), flush=True)


def _variant_errors(wl, grids, Q, dev):
    """FP32 / BF16 storage against FP64 storage on the same q: eigenvalue
    max and RMS error (meV) and eigenvector overlap loss 1 - |<v64, v>| over
    all (q, mode)."""
    import torch

    B, na = wl["w"].shape[1], wl["v"].shape[2]
    n = len(Q)
    Qd = torch.from_numpy(Q).to(dev)
    out = {}
    for st, g in grids.items():
        v = torch.empty((n, B), dtype=torch.float64, device=dev)
        c = torch.empty((n, B, na, 3), dtype=torch.complex128, device=dev)
        g.query_into(Qd, n, v, c)
        out[st] = (v, c)
    v64, c64 = out["f64"]
    res = {}
    for st in grids:
        if st == "f64":
            continue
        v, c = out[st]
        dv = (v - v64).abs()
        ov = (torch.conj(c64) * c).sum(dim=(2, 3)).abs() / (
            torch.linalg.vector_norm(c64, dim=(2, 3)) * torch.linalg.vector_norm(c, dim=(2, 3))).clamp_min(1e-300)
        e = 1 - ov
        res[st] = dict(eig_max_abs_meV=float(dv.max()), eig_rms_meV=float((dv ** 2).mean().sqrt()),
                       overlap_loss_max=float(e.max()), overlap_loss_mean=float(e.mean()),
                       overlap_loss_p999=float(torch.quantile(e.flatten()[:1 << 24].float(), 0.999)), q=n)
    return res


def run_throughput(args):
    """The headline: ir_interpolate_at on the default workload at the
    reference's precision (FP64 vertex data, float64 eigenvalues and
    complex128 eigenvectors out), 1e7 q per step; outputs of one step do not
    fit in HBM, so each step streams its q through one output buffer in
    chunks.  FP32 and BF16 storage follow as extra fields, with their error
    against the FP64 outputs."""
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from brille_gb300 import BZTrellisQdc
    from brille_gb300.sharding import shard_range

    wl = build_workload(args.workload)
    B, na = wl["w"].shape[1], wl["v"].shape[2]
    qr = wl["q_range"]
    n_step = args.q_per_step or WORKLOADS[args.workload][3]
    # weak scaling: a global batch of world·n q, each rank its own slice
    q0, q1 = shard_range(world * n_step, rank, world)
    n = q1 - q0
    gen = torch.Generator(device=dev)
    gen.manual_seed(1000 + rank)
    Qs = [(torch.rand((n, 3), generator=gen, device=dev, dtype=torch.float64) * 2 - 1) * qr for _ in range(2)]
    stream = torch.cuda.Stream(dev)
    sp = stream.cuda_stream
    peaks = measured_peaks()
    peak = float(peaks["hbm_gbs"]) if peaks else 6800.0

    def measure(storage, out_f32, steps, warmup):
        """value, stage times and roofline of one storage precision."""
        grid = BZTrellisQdc(wl["bz"], trellis=wl["tr"], device=local)
        grid.fill(wl["w"], [1, 0, 0, 0, 3], wl["v"], [0, 3 * na, 0, 2, 1], storage=storage)
        _, bq_vals, bq_vecs = bytes_per_q(B, na, out_f32)
        free, _ = torch.cuda.mem_get_info(dev)
        # one output buffer within 75 % of the free memory (the rest:
        # per-chunk records, grouping and tuning scratch), as few chunks as
        # that allows, of equal size: every chunk groups its q by node anew,
        # so the per-group work grows with the number of chunks
        cap = int(max(1 << 16, 0.75 * (free - (4 << 30)) / (bq_vals + bq_vecs + 500)))
        nch = -(-n // cap)
        m = -(-n // nch)
        chunks = [(a, min(n, a + m)) for a in range(0, n, m)]
        fdt = torch.float32 if out_f32 else torch.float64
        cdt = torch.complex64 if out_f32 else torch.complex128
        vals = torch.empty((m, B), dtype=fdt, device=dev)
        vecs = torch.empty((m, B, na, 3), dtype=cdt, device=dev)

        def step(i):
            Q = Qs[i % 2]
            for a, b in chunks:
                grid.query_into(Q[a:b], b - a, vals, vecs, out_f32=out_f32, async_=True, stream=sp)

        tuned = None
        if args.tuning and storage == args.storage:
            grid.set_tuning([int(x) for x in args.tuning.split(",")])
            tuned = grid.tuning()
        elif not args.no_tune:
            t = time.time()
            tuned = grid.tune(Qs[0][:m], out_f32=out_f32, reps=2, stream=sp, values_out=vals, vectors_out=vecs)
            log(f"[setup] {storage}: gather budgets (KB, values/vectors) {tuned} in {time.time() - t:.1f}s")
        for i in range(warmup):
            step(i)
            grid.sync(sp)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        grid.profile(True)
        l0 = grid.launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with Clocks(local) as clk:
            torch.cuda.synchronize()
            ev0.record(stream)
            for i in range(steps):
                step(i)
            ev1.record(stream)
            grid.sync(sp)
            torch.cuda.synchronize()
        launches = grid.launch_count() - l0
        stage_ms, stage_q, stage_groups = grid.stage_times()
        grid.profile(False)
        ms = ev0.elapsed_time(ev1)
        if dist:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
            dist.barrier()
        names = ["locate", "grouping", "gather_values", "gather_vectors"]
        dom = int(np.argmax(stage_ms))
        per_q = {0: 24 + 4 * 8 + 8 * 12 + 40, 1: 16, 2: bq_vals, 3: bq_vecs}[dom]
        ach = per_q * stage_q / (stage_ms[dom] / 1e3) / 1e9 if stage_ms[dom] > 0 else 0.0
        # DRAM bytes (read + write) per launch of the dominant kernel, from an
        # ncu capture, scaled to this launch's q
        prof = PROFILED_TRAFFIC.get((args.workload, names[dom], storage))
        traffic = None
        if prof:
            per_launch_q = stage_q / max(1, steps * len(chunks))
            traffic = round(prof["bytes_per_q"] * per_launch_q)
        roof = dict(bound="hbm", kernel=names[dom], achieved=round(ach, 1), peak=peak,
                    peak_source="measured" if peaks else "fallback", unit="GB/s", frac=round(ach / peak, 4),
                    traffic=traffic, traffic_source=prof["source"] if prof else None,
                    algorithmic_bytes_per_q=per_q, q_per_group=round(stage_q / max(stage_groups, 1), 2),
                    stage_ms_per_step={k: round(v / steps, 3) for k, v in zip(names, stage_ms)})
        fp = PROFILED_FP64.get((args.workload, names[dom], storage))
        if fp and stage_ms[dom] > 0:
            # the FP64 pipe bounds this kernel: its FP64 instructions per q
            # (ncu) over its measured time, against the pipe's issue rate
            sms = torch.cuda.get_device_properties(dev).multi_processor_count
            mhz = clk.summary().get("sm_mhz") or 2070.0
            qpg = stage_q / max(stage_groups, 1)
            ops_q = fp["per_q"] + fp["per_group"] / max(qpg, 1.0)
            rate = ops_q * stage_q / (stage_ms[dom] / 1e3)
            pk = sms * fp["lanes_per_sm_cycle"] * mhz * 1e6
            roof["fp64_pipe"] = dict(achieved_ops_per_s=rate, peak_ops_per_s=pk, frac=round(rate / pk, 4),
                                     ops_per_q=round(ops_q, 1), source=fp["source"])
        res = dict(value=world * n * steps / (ms / 1e3), ms_per_step=ms / steps, roofline=roof,
                   gpu_launches=int(launches), clocks=clk.summary(), chunk_q=m, chunks=len(chunks),
                   tuning=None if tuned is None else dict(
                       zip(("values_smem_kb", "vectors_smem_kb", "q_per_group", "units_per_thread", "gather_kernel"),
                           tuned)))
        return grid, vals, vecs, res

    out_f32 = args.storage != "f64" if args.out is None else args.out == "f32"
    grid, vals, vecs, main = measure(args.storage, out_f32, args.steps, args.warmup)
    _, bq_vals, bq_vecs = bytes_per_q(B, na, out_f32)

    # end to end through the public API: Q from pinned host memory, outputs
    # into a ring of two pinned host buffers that the step's calls fill in
    # turn (the outputs of 1e7 q, 373 GB at FP64, do not fit in host memory
    # either).  The calls are asynchronous (BRX_FLAG_ASYNC with page-locked
    # buffers), so one call's copies run on while the next one computes; a
    # buffer is refilled once the event behind its previous call has passed.
    # BRX_HOST_CHUNK_MB sets the library's staging chunk.
    e2e = None
    if args.e2e_steps > 0:
        del vals, vecs
        torch.cuda.empty_cache()
        host_gb = args.e2e_host_gb
        mh = int(min(n, host_gb * 1e9 / 2 / (bq_vals + bq_vecs)))
        # one staging chunk per call: the FP64 gather shares its per-group
        # work among the q of a group, and a larger chunk has more per group
        os.environ.setdefault("BRX_HOST_CHUNK_MB", str(max(512, min(65536, int(host_gb * 1e3 / 2 / 1.048576) + 1))))
        fdt = torch.float32 if out_f32 else torch.float64
        cdt = torch.complex64 if out_f32 else torch.complex128
        Qh = torch.empty((n, 3), dtype=torch.float64, pin_memory=True)
        Qh.copy_(Qs[0].cpu())
        vh = [torch.empty((mh, B), dtype=fdt, pin_memory=True) for _ in range(2)]
        ch = [torch.empty((mh, B, na, 3), dtype=cdt, pin_memory=True) for _ in range(2)]
        calls = [(a, min(n, a + mh)) for a in range(0, n, mh)]
        es = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]  # one per output buffer
        # the host link alone: a device buffer of one staging chunk copied to
        # each pinned output buffer in turn, sampled before every e2e step.
        # The first copy after the link has idled pays a wake-up cost (tens
        # to hundreds of ms); the copy right after it runs at the link's
        # sustained rate, which is what bounds the streaming e2e steps
        probe_bytes = min(int(os.environ["BRX_HOST_CHUNK_MB"]) << 20, ch[0].numel() * ch[0].element_size())
        probe = torch.empty(probe_bytes, dtype=torch.uint8, device=dev)
        chb = [c.view(torch.uint8).reshape(-1)[:probe_bytes] for c in ch]
        link, link_cold = [], []

        def link_sample():
            torch.cuda.synchronize()
            for k, dst in enumerate(chb):
                t = time.perf_counter()
                with torch.cuda.stream(stream):
                    dst.copy_(probe, non_blocking=True)
                stream.synchronize()
                (link_cold if k == 0 else link).append(probe_bytes / (time.perf_counter() - t) / 1e9)
            # the other buffer once more, now that the link is awake
            t = time.perf_counter()
            with torch.cuda.stream(stream):
                chb[0].copy_(probe, non_blocking=True)
            stream.synchronize()
            link.append(probe_bytes / (time.perf_counter() - t) / 1e9)

        def e2e_step():
            done = [None, None]
            for k, (a, b) in enumerate(calls):
                sl = k % 2
                if done[sl] is not None:
                    done[sl].synchronize()
                grid.query_into(Qh[a:b], b - a, vh[sl], ch[sl], out_f32=out_f32, async_=True,
                                stream=es[sl].cuda_stream)
                done[sl] = torch.cuda.Event()
                done[sl].record(es[sl])
            grid.sync()

        # freshly pinned pages reach full link speed only after a few passes
        for _ in range(2):
            link_sample()
        e2e_step()
        step_s = []
        for _ in range(args.e2e_steps):
            link_sample()
            if dist:
                dist.barrier()
            ts = time.perf_counter()
            e2e_step()
            step_s.append(time.perf_counter() - ts)
        while len(link_cold) < 5:
            link_sample()
        te = float(np.sum(step_s))
        if dist:
            t = torch.tensor([te], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            te = float(t.item())
        d2h = n * (bq_vals + bq_vecs)
        gbs = float(np.median(link[4:]))
        e2e = dict(value=world * n * args.e2e_steps / te, unit="q-points/s", h2d_bytes_per_step=n * 24,
                   d2h_bytes_per_step=d2h, q_per_step=n, calls_per_step=len(calls), host_buffer_q=mh,
                   host_buffers=2, staging_chunk_mb=int(os.environ["BRX_HOST_CHUNK_MB"]),
                   step_ms=[round(x * 1e3, 1) for x in step_s],
                   d2h_copy_gbs_median=round(gbs, 1), d2h_copy_gbs_samples=[round(x, 1) for x in link[4:]],
                   d2h_copy_gbs_after_idle=[round(x, 1) for x in link_cold[2:]],
                   d2h_copy_note="median of copies into both output buffers right after a first copy "
                                 "(the link's sustained rate); after_idle: that first copy",
                   d2h_copy_bound=round(world * gbs * 1e9 / (bq_vals + bq_vecs), 1),
                   frac_of_copy_bound=round((world * n * args.e2e_steps / te) / (world * gbs * 1e9 / (bq_vals + bq_vecs)),
                                            3))
        del probe, chb, vh, ch, Qh
    del grid
    torch.cuda.empty_cache()

    # reduced-precision storage: throughput and error against FP64
    variants = {}
    if not args.no_variants and args.storage == "f64" and world == 1:
        sub = np.random.default_rng(99).uniform(-qr, qr, size=(100_000, 3))
        errs_grids = {}
        for st in ("f32", "bf16"):
            g, vv, cc, r = measure(st, True, max(2, args.steps // 2), 3)
            del vv, cc
            r.pop("clocks", None)
            variants[st] = dict(value=r["value"], ms_per_step=r["ms_per_step"], outputs="f32/c64",
                                roofline=r["roofline"], gpu_launches=r["gpu_launches"], tuning=r["tuning"])
            errs_grids[st] = g
            torch.cuda.empty_cache()
        g64 = BZTrellisQdc(wl["bz"], trellis=wl["tr"], device=local)
        g64.fill(wl["w"], [1, 0, 0, 0, 3], wl["v"], [0, 3 * na, 0, 2, 1], storage="f64")
        errs_grids["f64"] = g64
        errs = _variant_errors(wl, errs_grids, sub, dev)
        for st in errs:
            variants[st]["error_vs_f64"] = errs[st]
        del errs_grids, g64
        torch.cuda.empty_cache()

    # the metric's own comparison: learned residual on coarse trellises
    # against plain trellises of increasing density (eigenvalues, 2e6
    # held-out q here; --mode learned runs 1e7)
    learned = None
    if not args.no_learned and world == 1:
        lc = learned_curve(args, 2_000_000, 3, 3)
        best = max(lc["learned"], key=lambda r: r.get("ratio_at_matched_max_error", r.get("ratio_vs_finest_plain", 0)))
        learned = dict(
            ratio_at_matched_max_error=best.get("ratio_at_matched_max_error"),
            ratio_at_matched_rms_error=best.get("ratio_at_matched_rms_error"),
            matched_plain_rms=best.get("matched_plain_rms"),
            learned=dict((k, best[k]) for k in ("trellis", "vertices", "max_meV", "rms_meV", "q_per_s")),
            matched_plain=best.get("matched_plain"),
            target=lc["target"], target_met=lc["target_met"],
            plain_vertices_for_1e_3_meV_max_extrapolated=lc["plain_max_error_fit"]["vertices_for_1e_3_meV"],
            plain_curve=[dict((k, c[k]) for k in ("trellis", "vertices", "max_meV", "rms_meV", "q_per_s"))
                         for c in lc["plain_curve"]],
            learned_all=[dict((k, r[k]) for k in ("trellis", "vertices", "max_meV", "rms_meV", "q_per_s"))
                         for r in lc["learned"]],
            crystal=lc["crystal"], q_eval=lc["q_eval"], exact=lc["exact"])
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(wl)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if rank == 0:
        f64 = args.storage == "f64" and not out_f32
        out = dict(
            metric=METRIC, value=main["value"], unit="q-points/s", n_gpus=world, steps=args.steps,
            warmup=args.warmup, ms_per_step=main["ms_per_step"], higher_is_better=True, scaling="weak",
            vs_baseline=None,
            dtype="f64" if f64 else "f64 predicates, f32 gather/rotate",
            data="synthetic (seeded BvK model at trellis vertices, q uniform)",
            config=dict(workload=args.workload, path="plain fine trellis, ir_interpolate_at",
                        trellis_vertices=int(len(wl["tr"].vertices)), modes=int(B), atoms=int(na),
                        trellis_build_s=wl["build_s"],
                        q_per_step=n, q_range=qr, storage=args.storage,
                        outputs="f32/c64" if out_f32 else "f64/c128",
                        chunk_q=main["chunk_q"], chunks_per_step=main["chunks"],
                        l2="outputs of %.1f GB per step, streamed through HBM; far above the 129 MB L2"
                           % (n * (bq_vals + bq_vecs) / 1e9),
                        tuning=main["tuning"],
                        parallelism=f"replicas x{world}, q sharded, no collective on the data path"),
            roofline=main["roofline"], e2e=e2e, cpu_baseline=cpu, gpu_launches=main["gpu_launches"],
            clocks=main["clocks"], variants=variants or None, learned=learned)
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hex16", choices=sorted(WORKLOADS))
    ap.add_argument("--q-per-step", type=int, default=0, help="default: the workload's batch")
    ap.add_argument("--storage", default="f64", choices=["f32", "f64", "bf16"])
    ap.add_argument("--out", default=None, choices=["f32", "f64"],
                    help="output precision (default: f64 for FP64 storage, else f32)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true", help="skip the FP32 / BF16 storage fields")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-vs-plain comparison")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--e2e-host-gb", type=float, default=64.0,
                    help="pinned host output buffers of the e2e calls (two, half each)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default gather shared-memory budgets")
    ap.add_argument("--tuning", default=None,
                    help="apply gather tuning values (5 integers, as config.tuning lists them) instead of tuning")
    ap.add_argument("--mode", default="throughput",
                    choices=["throughput", "precision", "learned", "batch", "sqw", "sort"],
                    help="precision: FP32 and BF16 storage against the FP64 path; learned: the learned residual "
                         "on coarse trellises against the plain fine trellis")
    ap.add_argument("--train-q", type=int, default=0, help="learned mode: training samples (default 1e6)")
    ap.add_argument("--epochs", type=int, default=30, help="learned mode: training epochs")
    ap.add_argument("--batch-items", type=int, default=64, help="batch mode: interpolators")
    ap.add_argument("--batch-vmax", type=float, default=2e5, help="batch mode: largest target vertex count")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)
    if args.mode == "precision":
        return run_precision(args)
    if args.mode == "learned":
        return run_learned(args)
    if args.mode == "batch":
        return run_batch(args)
    if args.mode == "sqw":
        return run_sqw(args)
    if args.mode == "sort":
        return run_sort(args)
    return run_throughput(args)


if __name__ == "__main__":
    main()
