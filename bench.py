#!/usr/bin/env python
"""Benchmark of the GB300 mesh boolean on the large single-pair workload.

Workload: pair_large — two icospheres at subdivision 7 (163,842 vertices / 327,680 triangles each), every
vertex jittered radially by U(-0.5%, +0.5%), the second with radius 0.9, offset (0.4, 0.1, -0.2) and a
seeded random rotation, seed 1234. Weld factor 1e8: the reference's own default (1e5) makes its combine()
fail on this workload ("Attach point to triangle edge failed"), so the full pipeline is timed at the
finer quantum where it succeeds; the status parity at 1e5 is covered by the tests.

One step = prepare both meshes (LBVH build) + combine() (candidate search, tri-tri, re-triangulation,
weld, arrangement, loops, groups, sides, fetch compaction) with inputs resident in HBM. The metric is
candidate triangle pairs per second (the reference's tri-pair workload divided by the whole-boolean time)
and, beside it, meshes/s (booleans per second). Both arithmetic forms run: the FP32-filtered form (the
headline `value`) and the plain FP64 form (`fp64_form`).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU restatement of the reference path (the oracle port; the reference sources
are not present on the GPU host) on the same workload on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from solidboolean_gb300 import meshgen as mg  # noqa: E402

METRIC = "Boolean tri-pairs/s (candidate triangle pairs / whole-boolean time), exact topology"
UNIT = "tri-pairs/s"
WELD = 100000000
LEVEL = 7
SEED = 1234
WORKLOAD = ("pair_large: icosphere L7 x2 (163,842 v / 327,680 t each), radial jitter +-0.5%, second mesh "
            "r=0.9 offset (0.4,0.1,-0.2) randomly rotated, seed 1234, weld factor 1e8")


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world: int, local: int):
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group(backend=backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region"""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload():
    return mg.pair_large(SEED, LEVEL)


# algorithmic bytes per launch of the instrumented kernels (per unit x units; the leaf-order kernels run
# once per mesh, so their figure is the mean over the two meshes)
def kernel_bytes(name: str, st: dict, na: int, nb: int, nva: int, nvb: int) -> float:
    C, K = st["candidate_pairs"], st["intersecting_pairs"]
    F = st["cut_faces_first"] + st["cut_faces_second"]
    T = st["result_triangles"]
    P = st["new_points"]
    return {
        # candidate search: each first-mesh triangle reads its FP32 box (24 B) and the second mesh's node
        # and leaf boxes once (24 B per node/leaf), writes 8 B per candidate
        "k_broad": 24.0 * na + 24.0 * (2 * nb) + 8.0 * C,
        # tri-tri: 8 B pair id + 6 FP32 vertices (96 B) per candidate, 1 B flag, 48 B segment per hit
        "k_narrow": (8 + 96 + 1) * C + 48.0 * K,
        # re-triangulation: segments in (48 B per pair side), corners (72 B) and out points / triangles
        "k_faces": 2 * 48.0 * K + 72.0 * F + 48.0 * P + 12.0 * 2 * F * 5,
        # half-edge tables: read 12 B per triangle, write 3 x (8 B key + 4 B owner)
        "k_halfedges": (12 + 36) * float(T),
        # union-find: read the triangle, three key lookups (12 B) and twin lookups (12 B), parent writes
        "k_union": (12 + 3 * 12 + 3 * 12 + 8) * float(T),
        "k_uf_flatten": 8.0 * T,
        # reference leaf order, large-node phase: every level reads each triangle's state word and the
        # integer record fields it classifies and reduces (centre key on the split axis, box keys and
        # fixed-point centre: 80 B) and writes the state back (8 B); levels = ceil(log2(n / 1024)) + 1
        "k_rr_top": 0.5 * 88.0 * (na * rr_levels(na) + nb * rr_levels(nb)),
        # subtree phase: sorted member index and Morton position (8 B), the record fields per level (80 B,
        # about log2(1024 / 20) + 1 levels) and the final position (4 B)
        "k_rr_subtree": 0.5 * (na + nb) * (8.0 + 80.0 * 7 + 4.0),
        # records: three vertex indices (12 B), nine coordinates (72 B), the FP64 box (48 B); writes the
        # 96 B record, its structure-of-arrays copy (96 B) and the position and state words (8 B)
        "k_rr_elems": 0.5 * (na + nb) * (12.0 + 72.0 + 48.0 + 96.0 + 96.0 + 8.0),
    }.get(name, 0.0)


# the kernel the roofline is reported for (the longest of the boolean; its event pairs are the only ones
# inside the timed steps)
ROOFLINE_KERNEL = "k_rr_top"

# DRAM bytes per launch (read + write) of the kernels captured with ncu on this workload; the figures and
# the command are in profiles/kernels_pair_large_L7.txt
MEASURED_TRAFFIC = {"k_rr_top": 32.85e6, "k_rr_subtree": 35.58e6, "k_faces": 14.53e6, "k_broad": 19.56e6,
                    "k_union": 26.97e6, "k_refit": 40.79e6}


def rr_levels(n: int) -> int:
    """levels of the reference tree's large-node phase for n triangles (nodes above 1024 members split)"""
    levels = 1
    while n > 1024:
        n = (n + 1) // 2
        levels += 1
    return levels


def gpu_arm(args, rank, world, local, dist):
    import torch
    import solidboolean_gb300 as sbg
    from solidboolean_gb300 import build as sbbuild
    sbbuild.build()
    L = sbg.lib()
    L.sb_kernel_timing.argtypes = [ctypes.c_int]
    L.sb_kernel_timing_read.restype = ctypes.c_int
    L.sb_kernel_timing_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_uint64)]
    L.sb_kernel_timing_names.restype = ctypes.c_int
    L.sb_kernel_timing_names.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.sb_kernel_timing_select.argtypes = [ctypes.c_char_p]
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    va, fa, vb, fb = workload()
    nva, nvb, na, nb = len(va), len(vb), len(fa), len(fb)
    stream = torch.cuda.Stream(device=dev)
    tv = [torch.from_numpy(x).to(dev) for x in (va, vb)]
    tt = [torch.from_numpy(x.astype(np.int32)).to(dev) for x in (fa, fb)]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    def run_form(precision: str, steps: int, warmup: int, timed_kernel: str | None):
        opts = sbg.make_options(WELD, precision, "reference", stream.cuda_stream)
        hA, hB, hX = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        sbg._check(L.sb_mesh_create_device(tv[0].data_ptr(), nva, tt[0].data_ptr(), na, ctypes.byref(opts),
                                           ctypes.byref(hA)), "create A")
        sbg._check(L.sb_mesh_create_device(tv[1].data_ptr(), nvb, tt[1].data_ptr(), nb, ctypes.byref(opts),
                                           ctypes.byref(hB)), "create B")
        sbg._check(L.sb_boolean_create(hA, hB, ctypes.byref(opts), ctypes.byref(hX)), "boolean")
        stats = sbg.Stats()
        pair_stage = []  # per timed step: device time of the candidate search and the tri-tri tests

        def step():
            # fresh vertex upload marks both meshes unprepared; combine() then rebuilds both meshes'
            # acceleration structures (concurrently, on two streams) before the boolean itself
            sbg._check(L.sb_mesh_update_vertices_device(hA, tv[0].data_ptr(), ctypes.byref(opts)), "update A")
            sbg._check(L.sb_mesh_update_vertices_device(hB, tv[1].data_ptr(), ctypes.byref(opts)), "update B")
            code = sbg._check(L.sb_combine(hX, ctypes.byref(stats)), "combine")
            return code

        for _ in range(warmup):
            with torch.cuda.stream(stream):
                flush.zero_()
            step()
        torch.cuda.synchronize()

        def read_timing():
            out = {}
            buf = ctypes.create_string_buffer(4096)
            L.sb_kernel_timing_names(buf, 4096)
            for name in buf.value.decode().split(","):
                if not name:
                    continue
                tot, n = ctypes.c_double(), ctypes.c_uint64()
                L.sb_kernel_timing_read(name.encode(), ctypes.byref(tot), ctypes.byref(n))
                out[name] = (tot.value, n.value)
            L.sb_kernel_timing(0)
            L.sb_kernel_timing_select(None)
            return out

        times = []
        launches0 = L.sb_kernel_launches()
        if timed_kernel is not None:
            # inside the timed steps only the roofline kernel carries an event pair (each timed launch adds
            # two events to its stream; timing every kernel slowed the step by about 0.1 ms)
            L.sb_kernel_timing_select(ROOFLINE_KERNEL.encode())
            L.sb_kernel_timing(1)
        barrier(dist)
        torch.cuda.synchronize()
        codes = set()
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()  # L2 flush outside the timed interval
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            codes.add(step())
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            pair_stage.append(stats.stage_ms[0] + stats.stage_ms[1])
        torch.cuda.synchronize()
        barrier(dist)
        launches = L.sb_kernel_launches() - launches0
        kern = {}
        if timed_kernel is not None:
            kern_head = read_timing()
            # every instrumented kernel, over as many further steps (not part of the timed steps)
            L.sb_kernel_timing(1)
            for _ in range(steps):
                with torch.cuda.stream(stream):
                    flush.zero_()
                step()
            torch.cuda.synchronize()
            kern = read_timing()
            kern.update(kern_head)
        st = stats.as_dict()
        st["pair_stage_ms"] = statistics.mean(pair_stage) if pair_stage else 0.0
        # results for the parity self-check (host copies, outside the timed region)
        res = None
        if precision == "filtered":
            X = sbg.SolidBoolean.__new__(sbg.SolidBoolean)
            X._h = hX
            res = {"status": 1 if 0 in codes else 0, "cand": X.dump("candidates", np.uint32, 2).astype(np.int64),
                   "isect_pairs": X.dump("intersection_pairs", np.uint32, 2).astype(np.int64),
                   "isect_segs": X.dump("intersection_segments", np.float64, 6), "newv": X.resultVertices(),
                   "newt": X.dump("arrangement", np.uint32, 3).astype(np.int64),
                   "labels": X.dump("labels", np.int8, 1)}
            for op in ("union", "diff", "intersect"):
                res[op] = X.fetch(op).astype(np.int64)
            X._h = ctypes.c_void_p()
        L.sb_boolean_destroy(hX)
        L.sb_mesh_destroy(hA)
        L.sb_mesh_destroy(hB)
        return times, st, codes, launches, kern, res

    sampler = ClockSampler(local)
    # plain FP64 form first (untimed clocks), then the filtered form with clocks sampled
    t64, st64, _, _, _, _ = run_form("fp64", args.steps, args.warmup, None)
    sampler.start()
    t32, st32, codes, launches, kern, res = run_form("filtered", args.steps, args.warmup, "all")
    clocks = sampler.stop()

    # e2e through the public API with host buffers (pinned), host<->device copies inside the timed region
    pin = [torch.from_numpy(x).pin_memory() for x in (va, fa, vb, fb)]
    hv = [p.numpy() for p in pin]
    e2e_times = []
    d2h = 0
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        opts = sbg.make_options(WELD, "filtered", "reference")
        A = sbg.SolidMesh(opts)
        A.setVertices(hv[0])
        A.setTriangles(hv[1])
        B = sbg.SolidMesh(opts)
        B.setVertices(hv[2])
        B.setTriangles(hv[3])
        A.prepare()
        B.prepare()
        X = sbg.SolidBoolean(A, B, opts)
        X.combine()
        outs = [X.fetch(op) for op in ("union", "diff", "intersect")]
        verts = X.resultVertices()
        t1 = time.perf_counter()
        del X, A, B
        if it >= args.warmup:
            e2e_times.append(t1 - t0)
            d2h = sum(o.nbytes for o in outs) + verts.nbytes
    h2d = va.nbytes + vb.nbytes + fa.nbytes + fb.nbytes

    ms32 = statistics.mean(t32)
    ms64 = statistics.mean(t64)
    C = st32["candidate_pairs"]
    ms32_max = allmax(dist, ms32)
    total_pairs = allsum(dist, float(C))
    value = total_pairs / (ms32_max / 1e3)
    e2e_s = allmax(dist, statistics.mean(e2e_times))

    # batched workload: independent pairs of mixed subdivision levels through sb_batch_combine, host inputs,
    # statuses only (the per-pair results stay on the device side of each worker); wall time of the call
    batch = None
    if args.batch_pairs > 0:
        pairs = mg.batch(args.batch_pairs, SEED, 5)
        sbg.batch_combine(pairs[:64], workers=8, keep=False)  # warm-up: handles, streams, buffers
        t0 = time.perf_counter()
        statuses, _ = sbg.batch_combine(pairs, workers=0, keep=False)  # worker count tuned by the library
        t1 = time.perf_counter()
        batch = {"workload": f"{args.batch_pairs} pairs: icospheres of levels U{{1..5}}, scale U[0.5, 2], random "
                             "rotations, centre distance U[0.2, 0.9](r1 + r2), op U{union, intersect, diff}, seed "
                             f"{SEED}, weld factor 1e5",
                 "meshes_per_s": allsum(dist, float(len(pairs))) / allmax(dist, t1 - t0), "s_total": t1 - t0,
                 "workers": "tuned by the library (4, 8 or 16 from three 64-pair runs)",
                 "failed_pairs": int(np.count_nonzero(statuses != 0)),
                 "timing": "host wall time of one sb_batch_combine call, host inputs"}
        # the same pairs in the robustness mode (not the reference's behaviour: scale-relative point-on-edge
        # bound, finer weld quanta after a failure), reported beside the parity mode
        t0 = time.perf_counter()
        rstat, _ = sbg.batch_combine(pairs, workers=0, keep=False, robust=sbg.SB_ROBUST_ALL)
        t1 = time.perf_counter()
        batch["robust_mode"] = {"failed_pairs": int(np.count_nonzero(rstat != 0)),
                                "meshes_per_s": allsum(dist, float(len(pairs))) / allmax(dist, t1 - t0),
                                "flags": "SB_ROBUST_EDGE_TOLERANCE | SB_ROBUST_WELD_RETRY"}
        if rank == 0 and args.batch_cpu_pairs > 0:
            cores = os.cpu_count() or 1
            sample = pairs[:args.batch_cpu_pairs]
            cpu_v, cpu_st = cpu_batch_baseline(sample, cores)
            same = sum(1 for i, c in enumerate(cpu_st) if (c == 1) == (statuses[i] == 0))
            batch["cpu_baseline"] = {"meshes_per_s": cpu_v, "cores": cores, "kind": "port",
                                     "sample": f"the first {len(sample)} pairs, one oracle process per host core "
                                               "(spawn pool), each pair single-threaded like the reference"}
            batch["status_parity_vs_oracle"] = f"{same}/{len(sample)}"

    # differentiable workload: intersection of two level-5 icospheres (B offset by seeded N(0, 0.01^2)),
    # forward (combine) and adjoint (sb_adjoint with a unit gradient on every result vertex), CUDA events
    adj = None
    if args.adjoint:
        ua, ufa, ub, ufb, uoff = mg.diff_volume(SEED, 5)
        ub = ub + uoff
        dv = [torch.from_numpy(x).to(dev) for x in (ua, ub)]
        dt = [torch.from_numpy(x.astype(np.int32)).to(dev) for x in (ufa, ufb)]
        o5 = sbg.make_options(WELD, "filtered", "reference", stream.cuda_stream)
        h5 = [ctypes.c_void_p() for _ in range(3)]
        sbg._check(L.sb_mesh_create_device(dv[0].data_ptr(), len(ua), dt[0].data_ptr(), len(ufa), ctypes.byref(o5),
                                           ctypes.byref(h5[0])), "A5")
        sbg._check(L.sb_mesh_create_device(dv[1].data_ptr(), len(ub), dt[1].data_ptr(), len(ufb), ctypes.byref(o5),
                                           ctypes.byref(h5[1])), "B5")
        sbg._check(L.sb_boolean_create(h5[0], h5[1], ctypes.byref(o5), ctypes.byref(h5[2])), "X5")
        st5 = sbg.Stats()
        tf, tb = [], []
        ga, gb = torch.zeros_like(dv[0]), torch.zeros_like(dv[1])
        for it in range(args.warmup + args.steps):
            sbg._check(L.sb_mesh_update_vertices_device(h5[0], dv[0].data_ptr(), ctypes.byref(o5)), "u5")
            sbg._check(L.sb_mesh_update_vertices_device(h5[1], dv[1].data_ptr(), ctypes.byref(o5)), "u5")
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            sbg._check(L.sb_combine(h5[2], ctypes.byref(st5)), "combine5")
            e1.record(stream)
            gv = torch.ones((int(st5.result_vertices), 3), dtype=torch.float64, device=dev)
            ga.zero_()
            gb.zero_()
            torch.cuda.synchronize()
            e1b = torch.cuda.Event(enable_timing=True)
            e1b.record(stream)
            sbg._check(L.sb_adjoint(h5[2], gv.data_ptr(), ga.data_ptr(), gb.data_ptr(), stream.cuda_stream), "adj")
            e2.record(stream)
            e2.synchronize()
            if it >= args.warmup:
                tf.append(e0.elapsed_time(e1))
                tb.append(e1b.elapsed_time(e2))
        L.sb_boolean_destroy(h5[2])
        L.sb_mesh_destroy(h5[0])
        L.sb_mesh_destroy(h5[1])
        adj = {"workload": "intersection of two icospheres L5 (20,480 t each), r 1 and 0.85, offset (0.35, 0, 0), "
                           "B offsets N(0, 0.01^2) seed 1234, weld factor 1e8",
               "forward_ms": statistics.mean(tf), "adjoint_ms": statistics.mean(tb),
               "appended_vertices": int(st5.new_points)}
    # roofline for the dominant instrumented kernel
    peak, peak_kind = measured_peaks()
    dom = (ROOFLINE_KERNEL, kern[ROOFLINE_KERNEL]) if ROOFLINE_KERNEL in kern else None
    roof = None
    if dom is not None:
        name, (tot_ms, n) = dom
        avg_ms = tot_ms / max(n, 1)
        alg = kernel_bytes(name, st32, na, nb, nva, nvb)
        ach = alg / (avg_ms / 1e3) / 1e9 if avg_ms > 0 else 0.0
        roof = {"kernel": name, "bound": "hbm", "achieved": round(ach, 2), "peak": peak, "unit": "GB/s",
                "frac": round(ach / peak, 5), "peak_kind": peak_kind, "avg_launch_ms": round(avg_ms, 4),
                "algorithmic_bytes": alg, "traffic": MEASURED_TRAFFIC.get(name),
                "share_of_step": round(tot_ms / max(sum(t32), 1e-9), 4)}
    per_kernel = {k: {"ms_per_launch": round(v[0] / max(v[1], 1), 4), "launches": v[1]} for k, v in kern.items()}
    return {
        "value": value, "ms_per_step": ms32_max, "stats": st32, "stats_fp64": st64, "t64": ms64,
        "codes": sorted(codes), "launches": launches, "clocks": clocks, "roofline": roof,
        "per_kernel": per_kernel, "e2e_s": e2e_s, "h2d": h2d, "d2h": d2h, "res": res,
        "total_pairs": total_pairs, "sizes": (nva, na, nvb, nb), "batch": batch, "adjoint": adj,
    }


def _oracle_pair(item):
    va, fa, vb, fb = item
    from oracle import oracle
    return int(oracle.port().run(va, fa, vb, fb, 100000)["status"])


def cpu_batch_baseline(pairs, cores: int):
    """The batched workload's pairs through the oracle port on every host core (one process per core, a spawn
    pool: the parent already holds a CUDA context); returns pairs/s and the per-pair statuses."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    items = [(va, fa, vb, fb) for va, fa, vb, fb, _ in pairs]
    with ProcessPoolExecutor(max_workers=cores, mp_context=mp.get_context("spawn")) as ex:
        list(ex.map(_oracle_pair, items[:cores]))  # each process loads the library once
        t0 = time.perf_counter()
        st = list(ex.map(_oracle_pair, items, chunksize=4))
        t1 = time.perf_counter()
    return len(items) / (t1 - t0), st


def cpu_reference(steps: int, warmup: int, check_with=None):
    """Times the oracle port (the reference's algorithm restated, single-threaded like the reference)."""
    from oracle import oracle
    P = oracle.port()
    va, fa, vb, fb = workload()
    times, d = [], None
    for it in range(warmup + steps):
        t0 = time.perf_counter()
        d = P.run(va, fa, vb, fb, WELD)
        t1 = time.perf_counter()
        if it >= warmup:
            times.append(t1 - t0)
    C = len(d["cand"])
    return C / statistics.mean(times), statistics.mean(times), d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample-runs", type=int, default=2)
    ap.add_argument("--batch-pairs", type=int, default=4096, help="pairs of the batched workload (0: skip)")
    ap.add_argument("--batch-cpu-pairs", type=int, default=1024,
                    help="pairs of the batched workload timed through the oracle port on all host cores (0: skip)")
    ap.add_argument("--adjoint", type=int, default=1, help="time forward + adjoint on the differentiable workload")
    args = ap.parse_args()
    rank, world, local = dist_info()

    if args.impl == "reference":
        if rank != 0:
            return
        steps, warmup = max(1, min(args.steps, 5)), min(args.warmup, 1)
        v, s, _ = cpu_reference(steps, warmup)
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": steps, "warmup": warmup, "ms_per_step": s * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                                 "sample": f"{steps} full booleans of the workload (prepare x2 + combine + fetch)"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    dist = init_dist(world, local)
    r = gpu_arm(args, rank, world, local, dist)
    if rank != 0:
        return
    # CPU baseline on a bounded sample (the same workload, single-threaded like the reference)
    cpu_v, cpu_s, cpu_d = cpu_reference(args.cpu_sample_runs, 0)
    parity = None
    if r["res"] is not None:
        from parity import compare
        nva, na, nvb, nb = r["sizes"]
        bad = compare(cpu_d, r["res"], nva + nvb, WELD)
        parity = "exact" if not bad else {k: str(v) for k, v in bad.items()}
    st = r["stats"]
    C = st["candidate_pairs"]
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "precision": "fp32-filtered predicates, fp64 constructions",
                   "l2": "flushed between steps (256 MiB write outside the timed interval)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "candidate_pairs": C, "intersecting_pairs": st["intersecting_pairs"],
                   "result_triangles": st["result_triangles"], "status_codes": r["codes"]},
        "meshes_per_s": world / (r["ms_per_step"] / 1e3),
        "fp64_form": {"value": C / (r["t64"] / 1e3), "unit": UNIT, "ms_per_step": r["t64"],
                      "meshes_per_s": 1e3 / r["t64"]},
        "filter": {"sign_tests": st["sign_tests"], "sign_fallbacks": st["sign_fallbacks"],
                   "fallback_rate": st["sign_fallbacks"] / max(st["sign_tests"], 1),
                   "box_tests": st["box_tests"], "box_fallbacks": st["box_fallbacks"]},
        "stage_ms": [round(x, 4) for x in st["stage_ms"][:7]],
        "roofline": r["roofline"], "per_kernel": r["per_kernel"],
        "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"{args.cpu_sample_runs} full booleans of the workload on one host core "
                                   f"({cpu_s:.2f} s each)"},
        "e2e": {"value": r["total_pairs"] / r["e2e_s"], "unit": UNIT, "h2d_bytes_per_step": int(r["h2d"]),
                "d2h_bytes_per_step": int(r["d2h"]), "ms_per_step": r["e2e_s"] * 1e3},
        "parity_vs_oracle": parity,
        "clocks": r["clocks"], "gpu_launches": int(r["launches"]),
        "batch": r["batch"], "adjoint": r["adjoint"],
    }
    # last, so that a tail of the output shows it: both arithmetic forms side by side, for the whole boolean
    # and for the tri-pair stage (candidate search + tri-tri tests, device time between the stage events)
    s32, s64 = st["pair_stage_ms"], r["stats_fp64"]["pair_stage_ms"]
    line["forms"] = {
        "filtered": {"ms_per_step": round(r["ms_per_step"], 4), "tri_pairs_per_s": round(r["value"]),
                     "pair_stage_ms": round(s32, 4), "pair_stage_tri_pairs_per_s": round(C / (s32 / 1e3)),
                     "sign_fallback_rate": st["sign_fallbacks"] / max(st["sign_tests"], 1)},
        "fp64": {"ms_per_step": round(r["t64"], 4), "tri_pairs_per_s": round(C / (r["t64"] / 1e3)),
                 "pair_stage_ms": round(s64, 4), "pair_stage_tri_pairs_per_s": round(C / (s64 / 1e3))},
        "filtered_over_fp64": {"boolean": round(r["t64"] / r["ms_per_step"], 3),
                               "pair_stage": round(s64 / s32, 3) if s32 > 0 else None}}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
