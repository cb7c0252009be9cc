#!/usr/bin/env python
"""Benchmark of the block-sparse contraction path on one GB300.

Workload (the block-sparse matrix product TSpArrayD, N = 16384): tile sizes
drawn uniformly from [48, 256] per dimension (seeded; the last tile absorbs a
remainder below 48), block (I, J) filled with uniform[-1, 1) entries scaled by
exp(-|I-J|/4) and absent when that factor is below 1e-10, SparseShape
threshold 1e-8 for the operands and the result.  Synthetic data generated on
the device with the counter-based generator.

A step is one C("i,j") = A("i,k") * B("k,j") through tagpu_contract with the
operands resident in HBM: screening, pair list, and the emulated-FP64 GEMM
(exact bf16 digit slices on tcgen05) that writes the result tiles.  The metric
is nonzero-block TFLOP/s = 2 * sum over the tile-pair list of m*k*n per
second.  The operands (~1.7 GB each) are far larger than L2, so no flush is
needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
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

METRIC = "nonzero-block TFLOP/s at <=1e-12 rel err, emulated vs plain FP64; p50/p99 latency"
SLICE_PAIRS = {s: s * (s + 1) // 2 for s in range(2, 9)}


def workload(n=16384, seed=0, lo=48, hi=256, decay=4.0, cut=1e-10):
    rng = np.random.default_rng(seed)
    h = [0]
    while h[-1] < n:
        rem = n - h[-1]
        s = int(rng.integers(lo, hi + 1))
        if rem - s < lo:
            s = rem
        h.append(h[-1] + s)
    nt = len(h) - 1
    I, J = np.meshgrid(np.arange(nt), np.arange(nt), indexing="ij")
    scale = np.exp(-np.abs(I - J) / decay)
    scale[scale < cut] = 0.0
    return h, scale


def profiled_traffic(name):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary profiles/<name> (line `traffic_bytes_per_launch: N`), or None."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region; the raw samples go to
    $BENCH_OUT_DIR (default: the temporary directory)."""

    def __init__(self, device):
        self.p = None
        out_dir = os.environ.get("BENCH_OUT_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, f"clocks_{os.getpid()}.csv")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(device),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 8:
                    continue
                try:
                    sm.append(float(parts[0]))
                    smax.append(float(parts[1]))
                except ValueError:
                    continue
                for name, v in zip(names, parts[4:8]):
                    if v.lower() == "active":
                        reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def host_placement(arrays, device=0):
    """Where the e2e host buffers live: pages per NUMA node of each buffer
    (from /proc/self/numa_maps), the NUMA node of the GPU's PCI function,
    and the CPUs and memory nodes this process may use."""
    info = {"cpus": len(os.sched_getaffinity(0))}
    for k in ("enabled", "defrag"):
        try:
            with open(f"/sys/kernel/mm/transparent_hugepage/{k}") as f:
                info["thp_" + k] = f.read().strip()
        except OSError:
            pass
    try:
        for line in open("/proc/self/status"):
            if line.startswith("Mems_allowed_list:"):
                info["mems_allowed"] = line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        import torch
        pr = torch.cuda.get_device_properties(device)
        bus = "%04x:%02x:%02x.0" % (getattr(pr, "pci_domain_id", 0), pr.pci_bus_id,
                                    pr.pci_device_id)
        info["gpu_pci"] = bus
        with open(f"/sys/bus/pci/devices/{bus}/numa_node") as f:
            info["gpu_numa_node"] = int(f.read().strip())
    except Exception:
        pass
    try:
        ends = {}
        for line in open("/proc/self/maps"):
            lo_s, hi_s = line.split()[0].split("-")
            ends[int(lo_s, 16)] = int(hi_s, 16)
        maps = open("/proc/self/numa_maps").read().splitlines()
        out = []
        for arr in arrays:
            lo, hi = arr.ctypes.data, arr.ctypes.data + arr.nbytes
            nodes = {}
            for line in maps:
                parts = line.split()
                start = int(parts[0], 16)
                if start >= hi or ends.get(start, start) <= lo:
                    continue
                for tok in parts[2:]:
                    k, _, v = tok.partition("=")
                    if k.startswith("N") and k[1:].isdigit():
                        nodes[k] = nodes.get(k, 0) + int(v)
                    elif k == "kernelpagesize_kB":
                        nodes["page_kB"] = int(v)
            out.append(nodes)
        info["buffers"] = out
    except Exception:
        pass
    return info


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_sample(A_t, B_t, h, scale, seconds, threads, seed=0, keep=False):
    """Oracle (vendor-BLAS dgemm per tile pair) on a bounded sample of result
    tiles of the same contraction; returns (TFLOP/s, sample description,
    seconds) and, with keep, the oracle's tiles (selected ordinals, their
    offsets into the buffer, the buffer)."""
    import oracle as O
    fn = O.openblas_dgemm()
    thr = 1e-8
    nt = len(h) - 1
    sizes = np.diff(np.asarray(h))
    An, Bn = A_t["norms"].reshape(nt, nt), B_t["norms"].reshape(nt, nt)
    ks = sizes.astype(np.float32)
    cn, _ = O.shape_gemm(An, Bn, ks, 1.0, thr)
    offs, kidx = O.pairs(cn, thr, An, thr, Bn, thr)
    # per result tile flops
    tile_fl = np.zeros(nt * nt)
    for t in range(nt * nt):
        ks_t = kidx[offs[t]:offs[t + 1]]
        if len(ks_t):
            tile_fl[t] = 2.0 * sizes[t // nt] * sizes[t % nt] * sizes[ks_t].sum()
    rng = np.random.default_rng(seed)
    cand = np.flatnonzero(tile_fl > 0)
    rng.shuffle(cand)
    msz = nsz = ksz = sizes.astype(np.int64)
    L = O.lib()
    P = lambda a, ty: a.ctypes.data_as(ty)

    def run(sel):
        sel = np.asarray(sorted(sel), np.int64)
        res_off = np.full(nt * nt, -1, np.int64)
        pos = 0
        for t in sel:
            res_off[t] = pos
            pos += int(sizes[t // nt] * sizes[t % nt])
        cbuf = np.zeros(max(pos, 1))
        t0 = time.perf_counter()
        L.orc_contract_subset(nt, nt, nt, P(msz, O._i64p), P(nsz, O._i64p), P(ksz, O._i64p),
                              P(A_t["data"], O._f64p), P(A_t["offsets"], O._i64p), 0,
                              P(B_t["data"], O._f64p), P(B_t["offsets"], O._i64p), 0,
                              P(offs, O._i64p), P(kidx, O._i32p), 1.0, P(cbuf, O._f64p),
                              P(res_off, O._i64p), P(sel, O._i64p), len(sel), threads, fn)
        return sel, time.perf_counter() - t0, res_off, cbuf

    # calibrate on a small sample, then size the timed sample to `seconds`
    def take(budget):
        sel, acc = [], 0.0
        for t in cand:
            sel.append(t)
            acc += tile_fl[t]
            if acc >= budget:
                break
        return sel
    cal = take(threads * 2e9)
    csel, cdt, _, _ = run(cal)
    rate = tile_fl[csel].sum() / max(cdt, 1e-6)
    sel, dt, res_off, cbuf = run(take(rate * seconds))
    fl = tile_fl[sel].sum()
    desc = (f"{len(sel)} of {len(cand)} nonzero result tiles ({fl / tile_fl.sum() * 100:.2f}% "
            f"of the flops), per-pair {'OpenBLAS' if fn else 'oracle-loop'} dgemm, {threads} threads")
    if keep:
        return fl / dt / 1e12, desc, dt, (sel, res_off, cbuf)
    return fl / dt / 1e12, desc, dt


def errors_vs_oracle(packed, offsets, h, oracle_tiles):
    """Relative Frobenius error of a GPU result (packed tiles, per-ordinal
    offsets) against the oracle's tiles: over all checked tiles together,
    the largest over single tiles, and the largest per band of |i - j|."""
    sel, res_off, cbuf = oracle_tiles
    nt = len(h) - 1
    sizes = np.diff(np.asarray(h))
    num = den = 0.0
    worst = 0.0
    band = {}
    for t in sel:
        i, j = int(t) // nt, int(t) % nt
        m, n = int(sizes[i]), int(sizes[j])
        ref = cbuf[res_off[t]:res_off[t] + m * n]
        o = int(offsets[t])
        got = packed[o:o + m * n] if o >= 0 else np.zeros(m * n)
        d = float(np.dot(got - ref, got - ref))
        r = float(np.dot(ref, ref))
        num += d
        den += r
        if r > 0:
            e = (d / r) ** 0.5
            worst = max(worst, e)
            b = abs(i - j) // 10 * 10
            band[b] = max(band.get(b, 0.0), e)
    return {"rel_err": (num / den) ** 0.5 if den > 0 else 0.0, "max_tile_rel_err": worst,
            "tiles_checked": int(len(sel)),
            "max_tile_rel_err_by_band": {f"{b}-{b + 9}": band[b] for b in sorted(band)}}


def run_reference(args):
    """CPU reference arm: the oracle port (the reference cannot be built here),
    all host threads, bounded samples of the same workload."""
    ws, rank, local = dist_env()
    if ws > 1 and rank != 0:
        return
    import oracle as O
    from oracle import build as ob
    ob.build()
    h, scale = workload(args.n, args.seed)
    nt = len(h) - 1
    thr = 1e-8
    t0 = time.perf_counter()
    tr = O.TiledRange([h, h])
    A = O.make_array(tr, args.seed, 0, 0, tile_scale=lambda i: float(scale[i[0], i[1]]),
                     keep=lambda i: scale[i[0], i[1]] != 0, threshold=thr)
    B = O.make_array(tr, args.seed, 1, 0, tile_scale=lambda i: float(scale[i[0], i[1]]),
                     keep=lambda i: scale[i[0], i[1]] != 0, threshold=thr)

    def pack(X):
        offs = np.full(nt * nt, -1, np.int64)
        bufs, pos = [], 0
        for o in range(nt * nt):
            t = X.tiles.get(o)
            if t is not None:
                offs[o] = pos
                bufs.append(t.ravel())
                pos += t.size
        return {"data": np.concatenate(bufs), "offsets": offs, "norms": X.norms.ravel()}
    At, Bt = pack(A), pack(B)
    threads = os.cpu_count() or 1
    vals, desc = [], ""
    per_step = max(0.5, min(args.cpu_seconds, 20.0, 120.0 / max(1, args.steps + args.warmup)))
    for s in range(args.warmup + args.steps):
        v, desc, dt = cpu_sample(At, Bt, h, scale, per_step, threads, seed=s)
        if s >= args.warmup:
            vals.append((v, dt))
    v = statistics.median(x[0] for x in vals)
    ms = statistics.median(x[1] for x in vals) * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "TFLOP/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded, generated on the host)",
            "config": {"workload": f"block-sparse matmul TSpArrayD N={args.n}, tiles U[48,256], "
                                   "exp(-|I-J|/4) blocks, threshold 1e-8",
                       "sample": desc},
            "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "setup_s": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)


def tensor_roofline(mma, ms, kernel):
    """Roofline object of the emulated form's tensor work: the bf16 flops of
    the digit-slice MMAs issued (`mma_flops`) over a CUDA-event time `ms`."""
    _, bf16_peak, peak_kind = peaks()
    achieved = mma / (ms * 1e-3) / 1e12
    return {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
            "frac": achieved / bf16_peak, "traffic": None, "kernel": kernel,
            "peak_kind": f"{peak_kind} bf16 burst", "mma_flops_per_step": mma}


def _line(args, metric, value, unit, ms, cfg, extra):
    out = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded counter-based generator, on device)", "config": cfg}
    out.update(extra)
    print(json.dumps(out), flush=True)


def ccsd_spot_check(C, V, T, hv, ho, thr, count=2):
    """Result tiles R(a,b,i,j) recomputed on the CPU in numpy FP64 from the
    operand tiles fetched from the device: the sum over the (c,d) tiles present
    in both shapes of V(a,b,c,d) @ T(c,d,i,j).  Checks the emulated GEMM at
    sizes where the plain FP64 form would take minutes per step.  Returns the
    largest relative Frobenius error over the checked tiles (the smallest v
    tiles, so the check stays at a few seconds at v = 384)."""
    nv, no = len(hv) - 1, len(ho) - 1
    sv, so = np.diff(np.asarray(hv)), np.diff(np.asarray(ho))
    voff, toff, coff = V.tile_offsets(), T.tile_offsets(), C.tile_offsets()
    order = np.argsort(sv, kind="stable")
    a0, a1 = int(order[0]), int(order[min(1, nv - 1)])
    picks = [(a0, a1, 0, no - 1), (a1, a0, no - 1, 0)][:count]
    worst, checked = 0.0, 0
    for a, b, i, j in picks:
        o = ((a * nv + b) * no + i) * no + j
        if coff[o] < 0:
            continue
        acc = np.zeros((sv[a] * sv[b], so[i] * so[j]))
        for c in range(nv):
            for d in range(nv):
                ov = ((a * nv + b) * nv + c) * nv + d
                ot = ((c * nv + d) * no + i) * no + j
                if voff[ov] < 0 or toff[ot] < 0:
                    continue
                acc += V.tile(ov, (acc.shape[0], -1)) @ T.tile(ot, (-1, acc.shape[1]))
        got = C.tile(o, acc.shape)
        worst = max(worst, float(np.linalg.norm(got - acc) / max(np.linalg.norm(acc), 1e-300)))
        checked += 1
    return worst, checked


def run_secondary(args):
    """The other configurations: measured lines for the record, not the
    headline (the default run is the block-sparse N=16384 product)."""
    import tiledarray_gb300 as ta
    from tiledarray_gb300 import build as tb
    from tiledarray_gb300 import workloads as wl
    tb.build()
    w = ta.World(0)
    prec = ta.PRECISION_OZAKI if args.precision == "ozaki" else ta.PRECISION_FP64

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        ms = []
        for _ in range(steps):
            w.timer_start()
            fn()
            ms.append(w.timer_stop())
        return ms

    def err_vs_plain(C, c_idx, A, a_idx, B, b_idx):
        Cp, stp = ta.contract(w, c_idx, 1.0, A, a_idx, B, b_idx, precision=ta.PRECISION_FP64)
        x, y = C.download(), Cp.download()
        return float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300)), stp

    if args.workload == "dense":
        tr = ta.TiledRange([list(range(0, 2049, 128))] * 2)
        A, B = ta.DistArray(w, tr), ta.DistArray(w, tr)
        A.generate(args.seed, 0, 0, None, False)
        B.generate(args.seed, 1, 0, None, False)
        res = {}
        ms = timed(lambda: res.__setitem__("c", ta.contract(w, "i,j", 1.0, A, "i,k", B, "k,j",
                                                            precision=prec)), args.steps,
                   args.warmup)
        C, st = res["c"]
        err, stp = err_vs_plain(C, "i,j", A, "i,k", B, "k,j")
        m = statistics.median(ms)
        extra = {"rel_err_vs_plain_fp64": err, "plain_ms": stp["ms_total"],
                 "phases_ms": {k: st[k] for k in ("ms_shape", "ms_pairs", "ms_split", "ms_gemm")}}
        if prec == ta.PRECISION_OZAKI and st["mma_flops"]:
            extra["roofline"] = tensor_roofline(st["mma_flops"], st["ms_gemm"],
                                                "ozaki_gemm (bf16 digit-slice MMAs issued)")
        _line(args, "dense TFLOP/s", st["flops"] / m / 1e9, "TFLOP/s", m,
              {"workload": "dense TArrayD 2048^3, tiles 128", "precision": args.precision},
              extra)
    elif args.workload == "ccsd":
        hv, ho, vs, ts = wl.ccsd(v=args.v, seed=args.seed)
        thr = 1e-8
        w.threshold = thr
        V = ta.DistArray(w, ta.TiledRange([hv, hv, hv, hv]))
        V.generate(args.seed, 0, 0, vs, True, thr)
        # identity: V(a,b,c,d) T(c,d,i,j); transpose: T stored as (i,j,c,d), the
        # form of the reference's abcd example, folded into the GEMM loaders;
        # general: V read as (a,c,b,d), an explicit tile permutation into GEMM order
        if args.form == "transpose":
            T = ta.DistArray(w, ta.TiledRange([ho, ho, hv, hv]))
            T.generate(args.seed, 1, 0, np.ascontiguousarray(ts.transpose(2, 3, 0, 1)), True, thr)
            a_idx, b_idx = "a,b,c,d", "i,j,c,d"
        else:
            T = ta.DistArray(w, ta.TiledRange([hv, hv, ho, ho]))
            T.generate(args.seed, 1, 0, ts, True, thr)
            a_idx, b_idx = ("a,c,b,d" if args.form == "general" else "a,b,c,d"), "c,d,i,j"
        res = {}
        ms = timed(lambda: res.__setitem__("c", ta.contract(
            w, "a,b,i,j", 1.0, V, a_idx, T, b_idx, precision=prec)),
            args.steps, args.warmup)
        C, st = res["c"]
        extra = {"phases_ms": {k: st[k] for k in ("ms_shape", "ms_pairs", "ms_permute",
                                                  "ms_split", "ms_gemm")},
                 "pairs": st["pairs"], "flops_per_step": st["flops"],
                 "permtypes": [st["left_permtype"], st["right_permtype"]]}
        if prec == ta.PRECISION_OZAKI and st["mma_flops"]:
            extra["roofline"] = tensor_roofline(st["mma_flops"], st["ms_gemm"],
                                                "ozaki_gemm (bf16 digit-slice MMAs issued)")
        if st["left_permtype"] == 3 and st["ms_permute"] > 0:
            moved = 16.0 * V.info().elements
            extra["permute"] = {"bytes": moved, "GB_per_s": moved / st["ms_permute"] / 1e6,
                                "hbm_peak_GB_per_s": peaks()[0]}
        if not args.no_plain and prec == ta.PRECISION_OZAKI:
            err, stp = err_vs_plain(C, "a,b,i,j", V, a_idx, T, b_idx)
            extra.update({"rel_err_vs_plain_fp64": err, "plain_fp64_tflops":
                          st["flops"] / stp["ms_total"] / 1e9})
        if not args.no_cpu and args.form == "identity":
            t0 = time.perf_counter()
            err, nchk = ccsd_spot_check(C, V, T, hv, ho, thr)
            extra["spot_check_vs_cpu"] = {"tiles": nchk, "max_rel_err": err,
                                          "seconds": time.perf_counter() - t0}
        m = statistics.median(ms)
        _line(args, "ccsd-like 4-index nonzero-block TFLOP/s", st["flops"] / m / 1e9, "TFLOP/s",
              m, {"workload": f"R(a,b,i,j)=V({a_idx})*T({b_idx}) o=48 v={args.v}",
                  "precision": args.precision, "V_bytes": V.info().device_bytes}, extra)
    elif args.workload == "batched":
        import ctypes
        cases = wl.batched(args.count, args.seed)
        ops = []
        for x, (tsl, ka, kb) in enumerate(cases):
            A = ta.DistArray(w, ta.TiledRange([tsl[0], tsl[1], tsl[2]]))
            B = ta.DistArray(w, ta.TiledRange([tsl[2], tsl[3]]))
            A.generate(args.seed, 2 * x, 0, ka, True)
            B.generate(args.seed, 2 * x + 1, 0, kb, True)
            ops.append((A, B))
        def batch(precision, steps, warmup):
            bh = ctypes.c_void_p()
            w.check(w.L.tagpu_batch_create(w.h, ctypes.byref(bh)))
            outs = []
            opts = ta.ContractOpts(precision, args.slices, -1.0)
            for A, B in ops:
                ch = ctypes.c_void_p()
                w.check(w.L.tagpu_batch_add(bh, b"i,j,l", 1.0, A.h, b"i,j,k", B.h, b"k,l",
                                            ctypes.byref(opts), ctypes.byref(ch)))
                outs.append(ta.DistArray(w, _handle=ch))
            t0 = time.perf_counter()
            w.check(w.L.tagpu_batch_run(bh))   # plan + capture + first run
            plan_s = time.perf_counter() - t0
            bst = ta.ContractStats()
            w.check(w.L.tagpu_batch_stats(bh, ctypes.byref(bst)))
            ms = timed(lambda: w.check(w.L.tagpu_batch_run(bh)), steps, warmup)
            w.check(w.L.tagpu_batch_destroy(bh))
            return ms, bst, plan_s, outs

        ms, bst, plan_s, outs = batch(prec, args.steps, args.warmup)
        m = statistics.median(ms)
        extra = {"flops_per_step": bst.flops, "pairs": bst.pairs, "plan_and_capture_s": plan_s,
                 "latency_ms": {"p50": float(np.percentile(ms, 50)),
                                "p99": float(np.percentile(ms, 99))}}
        if prec == ta.PRECISION_OZAKI and bst.mma_flops:
            # the GEMM launches run inside the captured graph: the time is
            # the whole replay (frames, splits and GEMMs)
            extra["roofline"] = tensor_roofline(
                bst.mma_flops, m, "graph replay: ozaki_gemm MMAs issued over the whole replay "
                                  "(frame, split and GEMM launches)")
        if not args.no_plain and prec == ta.PRECISION_OZAKI:
            pms, _, _, pouts = batch(ta.PRECISION_FP64, 1, 1)
            x = np.concatenate([o.download() for o in outs])
            y = np.concatenate([o.download() for o in pouts])
            pm = statistics.median(pms)
            extra.update({"plain_fp64": {"value": bst.flops / pm / 1e9, "ms_per_step": pm,
                                         "unit": "TFLOP/s"},
                          "emulated_over_plain": pm / m,
                          "rel_err_vs_plain_fp64": float(np.linalg.norm(x - y) /
                                                         max(np.linalg.norm(y), 1e-300))})
        _line(args, "batched nonzero-block TFLOP/s (one graph replay per step)",
              bst.flops / m / 1e9, "TFLOP/s", m,
              {"workload": f"{args.count} x C(i,j,l)=A(i,j,k)*B(k,l), extents log-U[32,512], "
                           "tiles U[32,128], 30% dropout", "precision": args.precision}, extra)
    elif args.workload == "serve":
        run_serve(args, w, ta, wl, prec)
    w.close()


def run_serve(args, w, ta, wl, prec):
    """Poisson request stream over the block-sparse, ccsd-like and batched
    families at scales U[0.25,1]; operands pre-generated and resident; the
    server admits by footprint under a 150 GB budget.

    Operands come from a pool drawn once: block-sparse products at four
    scales, ccsd-like contractions at scales spread over [0.25, 1] and
    batched-family contractions.  A ccsd-like request whose footprint (digit
    bricks of V dominate) can never fit the budget exists as arrays with a
    shape but no storage and must come back rejected.  Requests pick a family
    (weights --mix) and then a pool entry of it uniformly.  A sample of the
    served results (those under 0.5 TFLOP) is checked against the plain FP64
    form after the stream.  --rate a,b,c sweeps the arrival rate: one stream
    of --requests requests per rate, each through a fresh server."""
    import threading
    rng = np.random.default_rng(args.seed)
    thr = 1e-8
    pool = {"blocksparse": [], "ccsd": [], "batched": []}
    for x in range(4):
        sc = rng.uniform(0.25, 1.0)
        h, scale = wl.blocksparse(int(16384 * sc) // 64 * 64, seed=100 + x)
        tr = ta.TiledRange([h, h])
        A, B = ta.DistArray(w, tr), ta.DistArray(w, tr)
        A.generate(100 + x, 0, 0, scale, True, thr)
        B.generate(100 + x, 1, 0, scale, True, thr)
        pool["blocksparse"].append(("i,j", A, "i,k", B, "k,j", f"blocksparse s={sc:.2f}"))
    budget = 150 * 10 ** 9
    for x, sc in enumerate(np.linspace(0.25, 1.0, 6)):
        o = max(8, int(48 * sc) // 4 * 4)
        hv, ho, vs, ts = wl.ccsd(o=o, v=int(384 * sc), seed=200 + x)
        V = ta.DistArray(w, ta.TiledRange([hv, hv, hv, hv]))
        T = ta.DistArray(w, ta.TiledRange([hv, hv, ho, ho]))
        v = int(384 * sc)
        # V's digit bricks alone: v^4 elements x 2 bytes x slices
        if v ** 4 * 2 * args.slices < budget:
            V.generate(200 + x, 0, 0, vs, True, thr)
            T.generate(200 + x, 1, 0, ts, True, thr)
        # else: never admitted (its footprint bound, from the extents, exceeds the
        # budget): the arrays exist without storage
        pool["ccsd"].append(("a,b,i,j", V, "a,b,c,d", T, "c,d,i,j", f"ccsd s={sc:.2f}"))
    for x, (tsl, ka, kb) in enumerate(wl.batched(8, seed=300)):
        A = ta.DistArray(w, ta.TiledRange([tsl[0], tsl[1], tsl[2]]))
        B = ta.DistArray(w, ta.TiledRange([tsl[2], tsl[3]]))
        A.generate(300 + x, 0, 0, ka, True)
        B.generate(300 + x, 1, 0, kb, True)
        pool["batched"].append(("i,j,l", A, "i,j,k", B, "k,l", "batched"))
    w.threshold = thr
    fams = ["blocksparse", "ccsd", "batched"]
    mix = np.asarray([float(x) for x in args.mix.split(",")])
    mix = mix / mix.sum()
    rates = [float(x) for x in str(args.rate).split(",")]

    def stream(rate, seed):
        """One Poisson stream of args.requests requests at `rate` per second
        through a fresh server; returns its measurements."""
        srng = np.random.default_rng(seed)
        srv = ta.Server(w, hbm_budget_bytes=budget, max_batch=32, precision=prec,
                        slices=args.slices)
        arrivals = np.cumsum(srng.exponential(1.0 / rate, args.requests))
        fam_pick = srng.choice(3, size=args.requests, p=mix)
        picks = [pool[fams[f]][int(srng.integers(0, len(pool[fams[f]])))] for f in fam_pick]
        ids, rejected = [None] * args.requests, {}
        t0 = time.perf_counter()
        submitted = [0]

        def submitter():
            for x in range(args.requests):
                dt = arrivals[x] - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                c, A, a, B, b, name = picks[x]
                try:
                    ids[x] = srv.submit(c, 1.0, A, a, B, b)
                except ta.TAGPUError as e:
                    key = f"{name}: status {e.status}"
                    rejected[key] = rejected.get(key, 0) + 1
                submitted[0] = x + 1

        # the clients take their results as they complete (in submission
        # order), so finished results do not pile up in HBM; a sample is kept
        # for the check against the plain form
        results, failures, kept = [], {}, []

        def collector():
            for x in range(args.requests):
                while submitted[0] <= x:
                    time.sleep(0.0005)
                if ids[x] is None:
                    continue
                try:
                    C, res = srv.wait(ids[x], 600000)
                except ta.TAGPUError as e:
                    # the request failed on the device side (its status and the
                    # server's message); the stream goes on
                    key = f"{picks[x][5]}: status {e.status}"
                    failures[key] = failures.get(key, 0) + 1
                    continue
                results.append(res)
                if res["status"] != 0:
                    key = f"{picks[x][5]}: status {res['status']}"
                    failures[key] = failures.get(key, 0) + 1
                elif len(kept) < args.check and res["flops"] < 5e11 and x % 7 == 0:
                    kept.append((x, C))
                    continue
                del C
        th = threading.Thread(target=submitter)
        tc = threading.Thread(target=collector)
        th.start()
        tc.start()
        th.join()
        tc.join()
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.stop()
        # each kept result against the plain FP64 form of the same contraction
        worst = 0.0
        for x, C in kept:
            c, A, a, B, b, _ = picks[x]
            Cp, _ = ta.contract(w, c, 1.0, A, a, B, b, precision=ta.PRECISION_FP64)
            y, z = C.download(), Cp.download()
            worst = max(worst, float(np.linalg.norm(y - z) / max(np.linalg.norm(z), 1e-300)))
            del Cp, C
        flops = sum(r["flops"] for r in results)
        return {"rate": rate, "tflops": flops / wall / 1e12, "wall_s": wall,
                "requests_per_s": len(results) / wall,
                "latency_ms": {"p50": st["p50_ms"], "p99": st["p99_ms"], "mean": st["mean_ms"]},
                "completed": st["completed"], "rejected": sum(rejected.values()),
                "rejected_by_kind": rejected, "failed": st["failed"], "failures": failures,
                "kernel_waves": st["batches"], "peak_admitted_bytes": st["peak_bytes"],
                "checked_vs_plain": {"requests": len(kept), "max_rel_err": worst},
                "ms_per_request": wall * 1e3 / max(1, len(results))}

    sweep = [stream(r, args.seed + 17 * k) for k, r in enumerate(rates)]
    top = sweep[-1]
    extra = {k: top[k] for k in ("latency_ms", "requests_per_s", "completed", "rejected",
                                 "rejected_by_kind", "failed", "failures", "kernel_waves",
                                 "peak_admitted_bytes", "checked_vs_plain")}
    if len(sweep) > 1:
        extra["sweep"] = [{k: r[k] for k in ("rate", "tflops", "requests_per_s", "latency_ms",
                                             "completed", "rejected", "failed",
                                             "checked_vs_plain")} for r in sweep]
    _line(args, "served nonzero-block TFLOP/s; p50/p99 latency", top["tflops"], "TFLOP/s",
          top["ms_per_request"],
          {"workload": f"{args.requests} Poisson requests at {top['rate']}/s"
                       + (f" (also at {', '.join(str(r) for r in rates[:-1])}/s, same count)"
                          if len(rates) > 1 else "")
                       + f", families block-sparse/ccsd-like/batched in proportion {args.mix}, "
                       "scales U[0.25,1] (ccsd-like at six scales over [0.25,1]), 150 GB "
                       "admission budget, one persistent served GEMM",
           "precision": args.precision, "slices": args.slices}, extra)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="tagpu", choices=["tagpu", "reference"])
    ap.add_argument("--precision", default="ozaki", choices=["ozaki", "fp64"])
    ap.add_argument("--slices", type=int, default=7,
                    help="digit slices of the emulated form (7: 55-bit digits, every result "
                         "tile within 1e-12 of the oracle; 6: 47-bit, faster)")
    ap.add_argument("--alt-slices", type=int, default=6,
                    help="also time the emulated form at this slice count (0: no)")
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", default="blocksparse",
                    choices=["blocksparse", "dense", "ccsd", "batched", "serve"])
    ap.add_argument("--v", type=int, default=192, help="ccsd: virtual extent")
    ap.add_argument("--form", default="identity", choices=["identity", "transpose", "general"],
                    help="ccsd: operand index order (general = explicit tile permutation)")
    ap.add_argument("--count", type=int, default=512, help="batched: contractions")
    ap.add_argument("--requests", type=int, default=300, help="serve: requests")
    ap.add_argument("--rate", default="20", help="serve: Poisson arrivals / s; a comma list "
                    "sweeps the rates, one stream each (the last is the line's headline)")
    ap.add_argument("--mix", default="4,1,5",
                    help="serve: weights of the block-sparse, ccsd-like and batched families")
    ap.add_argument("--check", type=int, default=24,
                    help="serve: served results checked against the plain form")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    ws, rank, local = dist_env()
    if ws > 1:
        # The emulated GEMM loads shared A bricks with cluster-multicast bulk
        # copies; it runs only in single-GPU processes.  The path keeps every
        # contraction on one GPU and has no sharded form, so a multi-rank job
        # has nothing to measure.
        if rank == 0:
            print(json.dumps({"metric": METRIC, "n_gpus": ws, "skipped":
                              "single-GPU engine: the emulated GEMM uses cluster-multicast "
                              "loads and runs only in 1-GPU processes; no multi-GPU path"}),
                  flush=True)
        return 0
    if args.workload != "blocksparse":
        return run_secondary(args)
    local = 0
    import tiledarray_gb300 as ta
    from tiledarray_gb300 import build as tb
    tb.build()
    w = ta.World(local)
    thr = 1e-8
    w.threshold = thr
    h, scale = workload(args.n, args.seed)
    nt = len(h) - 1
    tr = ta.TiledRange([h, h])
    A = ta.DistArray(w, tr)
    B = ta.DistArray(w, tr)
    A.generate(args.seed, 0, 0, scale, True, thr)
    B.generate(args.seed, 1, 0, scale, True, thr)
    prec = ta.PRECISION_OZAKI if args.precision == "ozaki" else ta.PRECISION_FP64

    def step():
        C, st = ta.contract(w, "i,j", 1.0, A, "i,k", B, "k,j", precision=prec,
                            slices=args.slices)
        return C, st

    for _ in range(args.warmup):
        C, st = step()
        del C
    w.sync()
    clk = Clocks(local)
    ms_list, stats = [], None
    for _ in range(args.steps):
        w.timer_start()
        C, stats = step()
        ms_list.append(w.timer_stop())
        if _ != args.steps - 1:
            del C
    w.sync()
    clocks = clk.stop()
    total_ms = sum(ms_list)
    flops = stats["flops"]
    ms_step = total_ms / args.steps
    value = flops * args.steps / (total_ms * 1e-3) / 1e12
    lat = sorted(ms_list)
    p50 = float(np.percentile(lat, 50))
    p99 = float(np.percentile(lat, 99))
    hbm_peak, bf16_peak, peak_kind = peaks()
    pairs_per = SLICE_PAIRS.get(args.slices, 21) if prec == ta.PRECISION_OZAKI else 1
    gemm_ms = stats["ms_gemm"]
    if prec == ta.PRECISION_OZAKI:
        # the tensor work the GEMM issued: digit-slice MMAs over 128 x 64 x 32
        # stage blocks (padding of partial blocks included), fewer than
        # pairs_per per FP64 flop where digit shifts drop slice pairs
        mma = stats["mma_flops"] or flops * pairs_per
        achieved = mma / (gemm_ms * 1e-3) / 1e12
        roof = {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": achieved / bf16_peak, "traffic": None,
                "kernel": "ozaki_gemm (bf16 digit-slice MMAs issued; "
                          f"{mma / flops:.2f} bf16 flops per FP64 flop, {pairs_per} without "
                          "digit shifts)", "peak_kind": f"{peak_kind} bf16 burst",
                "mma_flops_per_step": mma,
                "fp64_equivalent": {"achieved": flops * pairs_per / (gemm_ms * 1e-3) / 1e12,
                                    "note": f"{pairs_per} slice products per FP64 product"}}
        if args.n == 16384 and args.slices == 7 and args.seed == 0:
            tb = profiled_traffic("ozaki_gemm_blocksparse_n8192_s7.md")
            if tb:
                roof["traffic"] = tb
                roof["traffic_note"] = (
                    "DRAM bytes per launch estimated from one ncu capture of the same "
                    "kernel at N=8192 scaled by the issued MMA work "
                    f"(profiles/ozaki_gemm_blocksparse_n8192_s7.md): "
                    f"{tb / (gemm_ms * 1e-3) / 1e9:.0f} GB/s over the timed GEMM = "
                    f"{tb / (gemm_ms * 1e-3) / 1e9 / hbm_peak:.2f} of {peak_kind} HBM")
    else:
        achieved = flops / (gemm_ms * 1e-3) / 1e12
        dmma_peak, _ = w.fp64_rates()
        roof = {"bound": "tensor", "achieved": achieved, "peak": dmma_peak,
                "unit": "TFLOP/s", "frac": achieved / dmma_peak, "traffic": None,
                "kernel": "dmma_gemm", "peak_kind": "measured DMMA rate (tagpu_device_fp64_rates)"}
    out = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64 (emulated: bf16 digit slices, exact int accumulation)"
           if prec == ta.PRECISION_OZAKI else "f64",
           "data": "synthetic (seeded counter-based generator, on device)",
           "config": {"workload": f"block-sparse matmul TSpArrayD N={args.n}, tiles U[48,256] "
                                  f"({nt} per dim), exp(-|I-J|/4) blocks cut at 1e-10, "
                                  "threshold 1e-8",
                      "precision": args.precision, "slices": args.slices if
                      prec == ta.PRECISION_OZAKI else None,
                      "pairs": stats["pairs"], "flops_per_step": flops,
                      "nonzero_result_tiles": stats["nonzero_result_tiles"],
                      "l2": "inputs larger than L2 (no flush)", "parallelism": "single GPU"},
           "latency_ms": {"p50": p50, "p99": p99},
           "phases_ms": {k: stats[k] for k in ("ms_shape", "ms_pairs", "ms_split", "ms_gemm")},
           "roofline": roof, "clocks": clocks,
           "gpu_launches": int(stats["kernel_launches"])}
    # results kept for the comparison with the oracle's tiles (CPU leg)
    kept_results = {"emulated" if prec == ta.PRECISION_OZAKI else "plain":
                    (C.download(), C.tile_offsets())}
    # the other slice count, timed the same way (its per-tile error is reported
    # beside the headline's)
    if prec == ta.PRECISION_OZAKI and args.alt_slices and args.alt_slices != args.slices:
        for _ in range(2):
            Ca, sta = ta.contract(w, "i,j", 1.0, A, "i,k", B, "k,j", precision=prec,
                                  slices=args.alt_slices)
            del Ca
        ams = []
        for _ in range(max(2, min(args.steps, 5))):
            w.timer_start()
            Ca, sta = ta.contract(w, "i,j", 1.0, A, "i,k", B, "k,j", precision=prec,
                                  slices=args.alt_slices)
            ams.append(w.timer_stop())
        am = statistics.median(ams)
        out["alt_slices"] = {"slices": args.alt_slices, "value": flops / (am * 1e-3) / 1e12,
                             "unit": "TFLOP/s", "ms_per_step": am, "ms_gemm": sta["ms_gemm"],
                             "mma_flops_per_step": sta["mma_flops"]}
        kept_results[f"emulated_S{args.alt_slices}"] = (Ca.download(), Ca.tile_offsets())
        del Ca
    # error vs plain FP64 (DMMA) on the device, and the plain form's speed
    if not args.no_plain and prec == ta.PRECISION_OZAKI:
        Cp, stp = ta.contract(w, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_FP64)
        x, y = C.download(), Cp.download()
        kept_results["plain"] = (y, Cp.tile_offsets())
        err = float(np.linalg.norm(x - y) / np.linalg.norm(y))
        dmma_peak, dfma_peak = w.fp64_rates()
        out["plain_fp64"] = {"value": flops / (stp["ms_total"] * 1e-3) / 1e12,
                             "ms_per_step": stp["ms_total"], "ms_gemm": stp["ms_gemm"],
                             "unit": "TFLOP/s", "dmma_peak_tflops": dmma_peak,
                             "dfma_peak_tflops": dfma_peak,
                             "frac_of_dmma_peak": flops / (stp["ms_gemm"] * 1e-3) / 1e12 /
                             dmma_peak}
        out["rel_err_vs_plain_fp64"] = err
        out["emulated_over_plain"] = value / out["plain_fp64"]["value"]
        imma, hmma = w.mma_sync_rates()
        out["mma_sync_rates"] = {"int8_tops": imma, "bf16_tflops": hmma,
                                 "note": "warp-level mma.sync paths of this GPU (measured); "
                                         "the emulated form runs on tcgen05 bf16"}
        del Cp, x
    # end to end through the public API with host buffers
    if not args.no_e2e:
        # pinned host buffers from the library (tagpu_host_alloc)
        a_host = w.host_array(A.info().elements)
        b_host = w.host_array(B.info().elements)
        a_host[:] = A.download()
        b_host[:] = B.download()
        c_host = None
        C2, _ = step()   # the result's pinned host buffer is allocated outside the timing
        c_host = w.host_array(C2.info().elements)
        del C2
        e2e_ms, parts = [], []
        iters = []
        # untimed warm-up passes over the same host buffers first (the first
        # touches of a fresh host buffer by the GPU ran slowly on some boxes)
        nwarm = max(1, min(args.warmup, 3))
        for it in range(nwarm + max(1, min(args.steps, 3))):
            t0 = time.perf_counter()
            A.upload(a_host)
            ta_ = time.perf_counter()
            B.upload(b_host)
            t1 = time.perf_counter()
            C2, st2 = step()
            t2 = time.perf_counter()
            n = C2.info().elements
            w.check(w.L.tagpu_array_download(C2.h, c_host.ctypes.data_as(ta._f64p), n))
            t3 = time.perf_counter()
            iters.append([round((ta_ - t0) * 1e3, 2), round((t1 - ta_) * 1e3, 2),
                          round((t2 - t1) * 1e3, 2), round((t3 - t2) * 1e3, 2)])
            del C2
            if it < nwarm:
                continue
            e2e_ms.append((t3 - t0) * 1e3)
            parts.append(((t1 - t0) * 1e3, (t2 - t1) * 1e3, (t3 - t2) * 1e3))
        e = statistics.median(e2e_ms)
        pm = parts[e2e_ms.index(e)] if e in e2e_ms else parts[0]
        out["e2e"] = {"value": flops / (e * 1e-3) / 1e12, "unit": "TFLOP/s",
                      "h2d_bytes_per_step": int(a_host.nbytes + b_host.nbytes),
                      "d2h_bytes_per_step": int(c_host.nbytes), "ms_per_step": e,
                      "phases_ms": {"h2d": pm[0], "contract": pm[1], "d2h": pm[2]},
                      "warmup_iters": nwarm,
                      "iters_ms": iters,   # per pass (warm-up first): upload A, upload B,
                                           # contract, download
                      "host": host_placement([a_host, b_host, c_host])}
        # the host link itself, outside the timed region: one 2 GB-class copy
        # each way from the library buffer and from a torch-pinned buffer
        import torch
        link = {}
        dev_t = torch.empty(a_host.size, dtype=torch.float64, device="cuda")
        pin_t = torch.empty(a_host.size, dtype=torch.float64, pin_memory=True)
        pin_t.fill_(0.5)
        for name, host_t in (("library", torch.from_numpy(a_host)), ("torch_pinned", pin_t)):
            for rep in range(2):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                dev_t.copy_(host_t, non_blocking=True)
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                host_t.copy_(dev_t, non_blocking=True)
                torch.cuda.synchronize()
                t2 = time.perf_counter()
            link[name] = {"h2d_GBs": a_host.nbytes / (t1 - t0) / 1e9,
                          "d2h_GBs": a_host.nbytes / (t2 - t1) / 1e9}
        t0 = time.perf_counter()
        A.upload(a_host)
        link["upload_A_ms_after"] = (time.perf_counter() - t0) * 1e3
        out["e2e"]["host_link"] = link
        del dev_t, pin_t
        if not args.no_cpu:
            A_t = {"data": a_host, "offsets": A.tile_offsets(), "norms": A.norms()}
            B_t = {"data": b_host, "offsets": B.tile_offsets(), "norms": B.norms()}
            threads = os.cpu_count() or 1
            v, desc, dt, otiles = cpu_sample(A_t, B_t, h, scale, args.cpu_seconds, threads,
                                             keep=True)
            out["cpu_baseline"] = {"value": v, "unit": "TFLOP/s", "cores": threads,
                                   "kind": "port", "sample": desc, "seconds": dt}
            # both GPU forms against the oracle's per-pair FP64 dgemm tiles
            out["vs_oracle"] = {k: errors_vs_oracle(pk, po, h, otiles)
                                for k, (pk, po) in kept_results.items()}
            del otiles
    print(json.dumps(out), flush=True)
    del A, B, C, kept_results
    w.close()


if __name__ == "__main__":
    main()
