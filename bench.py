#!/usr/bin/env python3
"""Throughput of brille's ir_interpolate_at query path on GB300.

One step = one ir_interpolate_at pass over one batch of seeded synthetic q
(uniform in [-L, L]³ r.l.u.) on the workload's trellis.  Default workload:
P6₃/mmc, a = 3.2 Å, c = 5.2 Å, 16 atoms (48 modes), eigenvalues plus
Γ-rotated eigenvectors, FP64 predicates, FP32 gather/rotate with
float32/complex64 outputs, q in [-2, 2]³.

Reported (one JSON line from rank 0):
  value      q-points/s, all ranks, inputs and outputs resident in HBM
  e2e        the same through the public API with pinned host Q and outputs
             (host→device and device→host copies inside the timed region)
  roofline   the dominant kernel's algorithmic bytes over its CUDA-event time
             against the measured HBM copy bandwidth
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


# dram__bytes_read.sum + dram__bytes_write.sum of one full-size launch (ncu,
# one pass, --clock-control none), keyed by (workload, stage)
PROFILED_TRAFFIC = {
    ("hex16", "gather_vectors"): dict(bytes=12_696_951_552 + 184_570_256_896,
                                      source="ncu, one full-size warp_gather_kernel launch"),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def build_workload(name):
    from brille_gb300 import workloads as W
    from brille_gb300.bz import BrillouinZone
    from brille_gb300.trellis import TrellisBuild

    builder, fraction, qr, _ = WORKLOADS[name]
    lat, masses = getattr(W, builder)()
    bz = BrillouinZone(lat)
    t = time.time()
    tr = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * fraction)
    log(f"[setup] trellis {tr.summary()} in {time.time() - t:.1f}s")
    model = W.bvk_for(lat, masses)
    qv = tr.vertices @ np.linalg.inv(lat.B)
    t = time.time()
    procs = min(16, os.cpu_count() or 1)
    w, v = model.modes(qv, chunk=2048, processes=procs if len(qv) > 8192 else 0)
    log(f"[setup] BvK modes for {len(qv)} vertices in {time.time() - t:.1f}s ({procs} processes)")
    return dict(name=name, lat=lat, bz=bz, tr=tr, model=model, w=w, v=v, q_range=qr)


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
    wl = build_workload(args.workload)
    vals = []
    import oracle.oracle as orc
    nthreads = orc.Oracle.max_threads()
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(wl, target_s=max(2.0, 60.0 / (args.steps + args.warmup)), threads=nthreads)
        if i >= args.warmup:
            vals.append(r)
    value = float(np.median([r["value"] for r in vals]))
    out = dict(metric="interp q-pts/s on 1 GB300 (learned+coarse vs plain GPU) at <=1e-3 meV max err",
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
    lat, _ = W.random_crystal(name, int(rng.integers(1, 7)), seed=seed, max_atoms=32)
    bz = BrillouinZone(lat)
    target = float(np.exp(rng.uniform(np.log(vmin), np.log(vmax))))
    ratio = bz.volume / ConvexHull(bz.ir_vertices_invA).volume
    frac = 4.0 / (ratio * target)
    tr = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * frac)
    # one correction: vertex count scales about as 1/node volume
    if not 0.67 < len(tr.vertices) / target < 1.5:
        tr = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * frac * len(tr.vertices) / target)
    return name, lat, tr


def run_batch(args):
    """64 interpolators of different space groups, trellises and mode counts,
    ragged q counts (log-uniform 1e3-5e6, 5e7 in all), values + Γ-rotated
    eigenvectors in FP32, answered by the batched path: one persistent launch
    per stage, autotuned, replayed from a captured CUDA graph.  All outputs
    of 5e7 q do not fit in HBM, so the q run in W waves of one graph replay
    each into reused output buffers."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    import torch

    from brille_gb300 import BZTrellisQdc
    from brille_gb300.batch import BatchQuery
    from brille_gb300.bz import BrillouinZone

    n_items = args.batch_items
    total_q = args.q_per_step or 50_000_000
    vmin, vmax = 2e3, args.batch_vmax
    t0 = time.time()
    procs = min(16, os.cpu_count() or 1)
    with ProcessPoolExecutor(max_workers=procs, mp_context=mp.get_context("spawn")) as ex:
        items = list(ex.map(_batch_item, range(n_items), [9000 + k for k in range(n_items)], [vmin] * n_items,
                            [vmax] * n_items))
    log(f"[batch] {n_items} trellises in {time.time() - t0:.1f}s")
    dev = torch.device("cuda")
    gen = torch.Generator(device=dev)
    gen.manual_seed(77)
    grids, B, na, V = [], [], [], []
    for name, lat, tr in items:
        bz = BrillouinZone(lat)
        nat = len(lat.basis.positions)
        nv, nb = len(tr.vertices), 3 * nat
        vals = torch.sort(torch.rand((nv, nb), generator=gen, device=dev) * 60.0, dim=1).values
        vecs = torch.randn((nv, nb, nat, 3), generator=gen, device=dev, dtype=torch.complex64)
        vecs /= torch.linalg.vector_norm(vecs, dim=(2, 3), keepdim=True)
        g = BZTrellisQdc(bz, trellis=tr)
        g.fill(vals, [1, 0, 0, 0, 3], vecs, [0, 3 * nat, 0, 2, 1], storage="f32")
        g._fill["values"] = g._fill["vectors"] = None  # the device copy is the handle's
        del vals, vecs
        grids.append(g)
        B.append(nb)
        na.append(nat)
        V.append(nv)
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
    with Clocks(0) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for w in range(waves):
            wave_io(w)
            bq.launch(sp)
            bq.sync(sp)  # the next set_io rewrites the pinned tables this replay reads
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = bq.launch_count() - l0
    # the same waves, one query per grid
    for i, g in enumerate(grids):
        if m[i]:
            g.query_into(Qall[i][:m[i]], m[i], vals[i], vecs[i], out_f32=True, stream=sp)
    torch.cuda.synchronize()
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev2.record(stream)
    for w in range(waves):
        for i, g in enumerate(grids):
            if m[i]:
                g.query_into(Qall[i][w * m[i]:(w + 1) * m[i]], m[i], vals[i], vecs[i], out_f32=True, async_=True,
                             stream=sp)
    ev3.record(stream)
    for g in grids:
        g.sync(sp)
    torch.cuda.synchronize()
    ms_single = ev2.elapsed_time(ev3)
    out_bytes = float((per_q * m).sum()) * waves
    peaks = measured_peaks()
    peak = float(peaks["hbm_gbs"]) if peaks else 6800.0
    achieved = out_bytes / (ms / 1e3) / 1e9
    out = dict(mode="batch", metric="interp q-pts/s, 64 interpolators batched", value=done_q / (ms / 1e3),
               unit="q-points/s", ms_total=ms, waves=waves, q_total=done_q, n_items=n_items,
               per_grid_queries=dict(value=done_q / (ms_single / 1e3), ms_total=ms_single,
                                     note="the same waves as one ir_interpolate_at call per grid, queued async"),
               speedup_vs_per_grid=ms_single / ms,
               config=dict(space_groups=list(BATCH_GROUPS), vertices=[int(min(V)), int(max(V)), int(np.median(V))],
                           modes=[int(min(B)), int(max(B))], atoms=[int(min(na)), int(max(na))],
                           q_per_item=[int(nq.min()), int(nq.max())], q_range=1.0, storage="f32",
                           outputs="f32 values + c64 Gamma-rotated eigenvectors",
                           data="synthetic random vertex data (sorted eigenvalues, unit eigenvectors), seeded",
                           tuned=cfg, graph="captured once, replayed per wave with new Q pointers"),
               roofline=dict(bound="hbm", kernel="whole batch (outputs only)", achieved=round(achieved, 1),
                             peak=peak, unit="GB/s", frac=round(achieved / peak, 4),
                             algorithmic_bytes=out_bytes, traffic=None),
               gpu_launches=int(launches), clocks=clk.summary())
    print(json.dumps(out), flush=True)


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


def run_learned(args):
    """Learned residual on coarse trellises of the 2-atom FCC crystal
    (a = 4.96 Å, 28 amu, BZ/5000 for the fine trellis) against the plain
    fine trellis: error against the exact BvK model on held-out uniform q in
    [-1,1]³, and eigenvalue throughput of each path on device-resident q."""
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

    def grid_at(frac):
        tr = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * frac)
        g = BZTrellisQdd(bz, trellis=tr)
        g.fill(model.frequencies(tr.vertices @ Binv)[:, :, None], [1, 0, 0, 0, 3], storage="f32")
        return g

    n_train = args.train_q or 1_000_000
    n_eval = args.q_per_step or 10_000_000
    t = time.time()
    Qt = np.random.default_rng(11).uniform(-1, 1, (n_train, 3))
    wt = model.frequencies(Qt, processes=procs)
    Qe = np.random.default_rng(12).uniform(-1, 1, (n_eval, 3))
    we = model.frequencies(Qe, processes=procs)
    log(f"[learned] exact BvK for {n_train} + {n_eval} q in {time.time() - t:.1f}s ({procs} processes)")
    Qd = torch.from_numpy(Qe).to(dev)
    Wd = torch.from_numpy(we).to(dev)
    out = torch.empty((n_eval, B), dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)
    sp = stream.cuda_stream

    def errors(g):
        g.query_into(Qd, n_eval, out, None, out_f32=True, stream=sp)
        torch.cuda.synchronize()
        e = (out.double() - Wd).abs()
        eh = e.cpu().numpy().ravel()
        return dict(max_meV=float(eh.max()), rms_meV=float(np.sqrt(np.mean(eh ** 2))),
                    p99_meV=float(np.quantile(eh, 0.99)), p9999_meV=float(np.quantile(eh, 0.9999)))

    def throughput(g):
        for _ in range(args.warmup):
            g.query_into(Qd, n_eval, out, None, out_f32=True, async_=True, stream=sp)
            g.sync(sp)
        torch.cuda.synchronize()
        g.profile(True)
        l0 = g.launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            g.query_into(Qd, n_eval, out, None, out_f32=True, async_=True, stream=sp)
        ev1.record(stream)
        g.sync(sp)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / args.steps
        st_ms, st_q, _ = g.stage_times()
        g.profile(False)
        return dict(q_per_s=n_eval / (ms / 1e3), ms_per_step=ms, gpu_launches=int(g.launch_count() - l0),
                    stage_ms_per_step=dict(zip(["locate", "grouping", "values", "vectors"],
                                               [round(x / args.steps, 3) for x in st_ms])))

    fine = grid_at(1 / 5000)
    res = dict(fine=dict(trellis="bz/5000", vertices=int(len(fine.trellis.vertices)), plain=errors(fine),
                         speed=throughput(fine)))
    peaks = measured_peaks()
    for name, frac in LEARNED_COARSE:
        g = grid_at(frac)
        r = dict(vertices=int(len(g.trellis.vertices)), plain=errors(g), plain_speed=throughput(g))
        m = ResidualModel(B, seed=0)
        torch.cuda.synchronize()
        t = time.time()
        hist = m.train_on(g, Qt, wt, epochs=args.epochs, batch=4096, lr=2e-3, log=log)
        torch.cuda.synchronize()
        r["train"] = dict(samples=n_train, epochs=args.epochs, batch=4096, seconds=round(time.time() - t, 2),
                          loss_first=hist[0], loss_last=hist[-1], params=m.n_params,
                          res_scale_meV=m.res_scale, clip_meV=m.clip)
        m.attach(g)
        r["learned"] = errors(g)
        r["learned_speed"] = sp_ = throughput(g)
        # the residual kernel runs inside the values stage: its share is the
        # difference to the plain coarse path
        mlp_ms = sp_["stage_ms_per_step"]["values"] - r["plain_speed"]["stage_ms_per_step"]["values"]
        flops_q = 2 * (m.d_in * 128 + 2 * 128 * 128 + 128 * m.n_out)
        if mlp_ms > 0:
            ach = flops_q * n_eval / (mlp_ms / 1e3) / 1e12
            peak = float(peaks["bf16_tflops"]) if peaks else 1900.0
            r["mlp_roofline"] = dict(bound="tensor", achieved=round(ach, 2), peak=peak, unit="TFLOP/s",
                                     frac=round(ach / peak, 4), flops_per_q=flops_q, ms_per_step=round(mlp_ms, 3),
                                     peak_source="measured" if peaks else "fallback")
        r["speedup_vs_fine"] = sp_["q_per_s"] / res["fine"]["speed"]["q_per_s"]
        res[name] = r
        log(f"[learned] {name}: plain max {r['plain']['max_meV']:.3g} rms {r['plain']['rms_meV']:.3g}; "
            f"learned max {r['learned']['max_meV']:.3g} rms {r['learned']['rms_meV']:.3g} meV; "
            f"{sp_['q_per_s']:.3g} q/s vs fine {res['fine']['speed']['q_per_s']:.3g}")
    out_line = dict(mode="learned", crystal="FCC Fd-3m a=4.96 A, 2-atom primitive basis, 28 amu, 6 modes",
                    q_eval=n_eval, q_eval_set="uniform in [-1,1]^3 r.l.u., seed 12 (held out)",
                    train_set="uniform in [-1,1]^3 r.l.u., seed 11, folded into the wedge by the locate",
                    exact="BvK eigenvalues (FP64 eigvalsh) at each q", outputs="f32 eigenvalues, storage f32",
                    target="<=1e-3 meV max error", steps=args.steps, warmup=args.warmup, results=res)
    print(json.dumps(out_line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hex16", choices=sorted(WORKLOADS))
    ap.add_argument("--q-per-step", type=int, default=0, help="default: the workload's batch")
    ap.add_argument("--storage", default="f32", choices=["f32", "f64", "bf16"])
    ap.add_argument("--out-f64", action="store_true", help="float64/complex128 outputs")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
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

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
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

    import torch

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
    grid = BZTrellisQdc(wl["bz"], trellis=wl["tr"], device=local)
    grid.fill(wl["w"], [1, 0, 0, 0, 3], wl["v"], [0, 3 * na, 0, 2, 1], storage=args.storage)
    out_f32 = not args.out_f64
    n = args.q_per_step or WORKLOADS[args.workload][3]
    bq_in, bq_vals, bq_vecs = bytes_per_q(B, na, out_f32)
    free, _ = torch.cuda.mem_get_info(dev)
    fit = int(0.85 * (free - (2 << 30)) / (bq_vals + bq_vecs + 2 * 24 + 2 * 200))
    if n > fit:
        log(f"[setup] {n} q per step do not fit in HBM; using {fit}")
        n = fit
    qr = wl["q_range"]
    # weak scaling: a global batch of world·n q, each rank its own slice
    q0, q1 = shard_range(world * n, rank, world)
    n = q1 - q0
    gen = torch.Generator(device=dev)
    gen.manual_seed(1000 + rank)
    nbuf = 2
    Qs = [(torch.rand((n, 3), generator=gen, device=dev, dtype=torch.float64) * 2 - 1) * qr for _ in range(nbuf)]
    fdt = torch.float32 if out_f32 else torch.float64
    cdt = torch.complex64 if out_f32 else torch.complex128
    vals = torch.empty((n, B), dtype=fdt, device=dev)
    vecs = torch.empty((n, B, na, 3), dtype=cdt, device=dev)
    stream = torch.cuda.Stream(dev)
    sp = stream.cuda_stream

    def step(i):
        grid.query_into(Qs[i % nbuf], n, vals, vecs, out_f32=out_f32, async_=True, stream=sp)

    tuned = None
    if args.tuning:
        grid.set_tuning([int(x) for x in args.tuning.split(",")])
        tuned = grid.tuning()
    elif not args.no_tune:
        t = time.time()
        tuned = grid.tune(Qs[0], out_f32=out_f32, reps=2, stream=sp, values_out=vals, vectors_out=vecs)
        log(f"[setup] gather budgets (KB, values/vectors) {tuned} in {time.time() - t:.1f}s")

    for i in range(args.warmup):
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
        for i in range(args.steps):
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
    ms_per_step = ms / args.steps
    value = world * n * args.steps / (ms / 1e3)

    # roofline of the dominant kernel
    stage_names = ["locate", "grouping", "gather_values", "gather_vectors"]
    dom = int(np.argmax(stage_ms))
    per_q_bytes = {0: bq_in + 4 * 8 + 8 * 12 + 40, 1: 16, 2: bq_vals, 3: bq_vecs}[dom]
    achieved = per_q_bytes * stage_q / (stage_ms[dom] / 1e3) / 1e9 if stage_ms[dom] > 0 else 0.0
    peaks = measured_peaks()
    peak = float(peaks["hbm_gbs"]) if peaks else 6800.0
    # DRAM bytes (read + write) of one launch of the dominant kernel on this
    # workload, from an ncu capture of the full-size launch
    prof = PROFILED_TRAFFIC.get((args.workload, stage_names[dom])) if n == WORKLOADS[args.workload][3] else None
    traffic = None
    if prof:
        traffic = dict(bytes_per_launch=prof["bytes"], algorithmic_bytes_per_launch=per_q_bytes * n,
                       ratio=round(prof["bytes"] / (per_q_bytes * n), 3), source=prof["source"])
    roofline = dict(bound="hbm", kernel=stage_names[dom], achieved=round(achieved, 1), peak=peak,
                    peak_source="measured" if peaks else "fallback", unit="GB/s",
                    frac=round(achieved / peak, 4), traffic=traffic,
                    algorithmic_bytes_per_q=per_q_bytes,
                    q_per_group=round(stage_q / max(stage_groups, 1), 2),
                    stage_ms_per_step={k: round(v / args.steps, 3) for k, v in zip(stage_names, stage_ms)})

    # end to end through the public API with pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        ne = min(n, 1 << 20)
        Qh = torch.empty((ne, 3), dtype=torch.float64, pin_memory=True)
        Qh.copy_(Qs[0][:ne].cpu())
        vh = torch.empty((ne, B), dtype=fdt, pin_memory=True)
        ch = torch.empty((ne, B, na, 3), dtype=cdt, pin_memory=True)
        # freshly pinned pages reach full link speed only after a few passes
        for _ in range(max(6, args.warmup)):
            grid.query_into(Qh, ne, vh, ch, out_f32=out_f32)
        t0 = time.perf_counter()
        step_s = []
        for _ in range(args.e2e_steps):
            ts = time.perf_counter()
            grid.query_into(Qh, ne, vh, ch, out_f32=out_f32)
            step_s.append(time.perf_counter() - ts)
        te = time.perf_counter() - t0
        if dist:
            t = torch.tensor([te], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            te = float(t.item())
        h2d = ne * 24
        d2h = ne * (bq_vals + bq_vecs)
        # the host link alone: the same output bytes copied device -> pinned host
        torch.cuda.synchronize()
        tl = time.perf_counter()
        with torch.cuda.stream(stream):
            ch.copy_(vecs[:ne], non_blocking=True)
            vh.copy_(vals[:ne], non_blocking=True)
        stream.synchronize()
        tl = time.perf_counter() - tl
        e2e = dict(value=world * ne * args.e2e_steps / te, unit="q-points/s", h2d_bytes_per_step=h2d,
                   d2h_bytes_per_step=d2h, step_ms=[round(x * 1e3, 1) for x in step_s],
                   d2h_copy_gbs=round(d2h / tl / 1e9, 1), d2h_copy_bound=round(world * ne / tl, 1))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(wl)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if rank == 0:
        out = dict(
            metric="interp q-pts/s on 1 GB300 (learned+coarse vs plain GPU) at <=1e-3 meV max err",
            value=value, unit="q-points/s", n_gpus=world, steps=args.steps, warmup=args.warmup,
            ms_per_step=ms_per_step, higher_is_better=True, scaling="weak", vs_baseline=None,
            dtype="f64 predicates, f32 gather/rotate" if args.storage != "f64" else "f64",
            data="synthetic (seeded BvK model at trellis vertices, q uniform)",
            config=dict(workload=args.workload, path="plain fine trellis, ir_interpolate_at",
                        trellis_vertices=int(len(wl["tr"].vertices)), modes=int(B), atoms=int(na),
                        q_per_step=n, q_range=qr, storage=args.storage,
                        outputs="f32/c64" if out_f32 else "f64/c128",
                        l2="outputs of %.1f GB per step exceed the 129 MB L2" % (n * (bq_vals + bq_vecs) / 1e9),
                        tuning=None if tuned is None else dict(
                            zip(("values_smem_kb", "vectors_smem_kb", "q_per_group", "units_per_thread",
                                 "gather_kernel"), tuned)),
                        parallelism=f"replicas x{world}, q sharded, no collective on the data path"),
            roofline=roofline, e2e=e2e, cpu_baseline=cpu, gpu_launches=int(launches),
            clocks=clk.summary())
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
