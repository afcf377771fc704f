#!/usr/bin/env python3
"""Benchmark of the Groth16/BN254 prover core on GB300: SquareChain(2^18) ms/proof.

Workload (one step = one complete proof, all five MSMs and the QAP NTTs): the seeded
synthetic SquareChain(2^18) instance (bend2/FORMAT.md files; N = 2^18 constraints,
d = 2^19 domain, n_a = n_b = 2^18+2, n_h = 2^19-1, n_l = 2^18), generated once per box and
cached.  No public dataset is involved; the instance has the shapes of the reference's K=18
runs (bend2/bench/prover_results.md:59).

  value  ms/proof with the proving key and the witness resident in HBM before timing
         (bg_pk_upload + a device copy of witness.bin), CUDA events on the library's stream,
         L2 flushed (512 MiB write) before every step outside the timed events.
  e2e    ms/proof through bg_prove_host with every .bin file in pinned host memory: the whole
         upload (all files), the proof and the result reads are inside the timed region.
  roofline  the dominant kernel's algorithmic 32-bit multiply-adds per launch over its
         CUDA-event duration, against the IMAD rate measured by the library's probe.
  cpu_baseline  the C restatement in oracle/ (the reference's Bend/Rust CPU paths cannot
         run here), all host threads, one proof of the same instance, rank 0 at N=1.

`--impl reference` times that CPU restatement alone (rank 0; other ranks exit 0).
Multi-GPU: replicas only (every rank proves its own copy; no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "bend-groth16_gb300")
sys.path.insert(0, PKG)

METRIC = "SquareChain 2^18 ms/proof"
UNIT = "ms/proof"
# the reference's own GPU path (Bend 2 CUDA, RTX 5090) at K=18, T total
# (bend2/bench/prover_results.md:63, README.md:57)
REF_GPU_K18_MS = 56083.0
# 32-bit multiply-adds (mad.lo + mad.hi) the accumulation kernel executes per mixed addition
# (madd-2008-s), from the products of fp_wide.cuh: a 512-bit Karatsuba product 3 x 32 = 96,
# a 512-bit square 72, a Montgomery reduction 8 x 17 = 136.  Fq product 232, square 208,
# u v - w z 2 x 96 + 136 = 328.  G1: 6 products + 2 squares + Y3 = 2136.  G2 (Fq2 product 3 x 96
# + 2 x 136 = 560, square = 2 Fq products, u v - w z 6 x 96 + 2 x 136 = 848): 6 x 560 +
# 2 x 464 + 848 = 5136.
MADD_G1_IMAD = 6 * (96 + 136) + 2 * (72 + 136) + (2 * 96 + 136)
MADD_G2_IMAD = 6 * (3 * 96 + 2 * 136) + 2 * 2 * (96 + 136) + (6 * 96 + 2 * 136)
# per affine pair addition of the batch-affine rounds (msm_pairs.cuh): three products of the
# shared inversion (running product, 1/d, and the inverse walked back), the slope, its square
# and y3: 5 products + 1 square.  G1: 5 x 232 + 208 = 1368; G2: 5 x 560 + 464 = 3264.
PAIR_G1_IMAD = 5 * (96 + 136) + (72 + 136)
PAIR_G2_IMAD = 5 * (3 * 96 + 2 * 136) + 2 * (96 + 136)
KERNEL_FAMILIES = ["msm_pair_g1", "msm_pair_g2", "msm_bucket_acc_g1", "msm_bucket_acc_g2", "msm_heavy_g1",
                   "msm_heavy_g2", "msm_reduce_g1", "msm_reduce_g2", "msm_digits", "msm_scatter", "ntt_pass"]


def bucket_counts(sc_u32, c: int):
    """entries per bucket key of one bucket set per window, for (n, 8) uint32 canonical scalars
    and window width c: the balanced window layout and signed digits of msm.cu (window_width,
    window_offset, signed_digit), key = w 2^(c-1) + |d| - 1"""
    import numpy as np
    W = 254 // c + 1
    nb = 1 << (c - 1)
    base, extra = 255 // W, 255 % W
    limbs = sc_u32.astype(np.uint64)
    carry = np.zeros(sc_u32.shape[0], dtype=np.uint64)
    counts = np.zeros(W * nb, dtype=np.int64)
    for w in range(W):
        b = base + (1 if w < extra else 0)
        off = w * base + min(w, extra)
        li, sh = off // 32, off % 32
        v = limbs[:, li].copy()
        if li + 1 < 8:
            v |= limbs[:, li + 1] << np.uint64(32)
        d = ((v >> np.uint64(sh)) & np.uint64((1 << b) - 1)) + carry
        neg = d > np.uint64(1 << (b - 1))
        mag = np.where(neg, np.uint64(1 << b) - d, d)
        carry = neg.astype(np.uint64)
        keys = (mag[mag > 0] - np.uint64(1)).astype(np.int64)
        counts[w * nb:(w + 1) * nb] += np.bincount(keys, minlength=nb)
    return counts


def pair_round_additions(counts, rounds: int):
    """affine additions of each batch-affine round: a bucket of m points gives floor(m / 2)
    sums and keeps ceil(m / 2) points for the next round"""
    m = counts.astype("int64")
    out = []
    for _ in range(rounds):
        out.append(int((m // 2).sum()))
        m = (m + 1) // 2
    return out


def parse():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--log2n", type=int, default=18)
    ap.add_argument("--seed", type=int, default=18181818)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-primitives", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-proof mixed-K batch measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the Poisson-arrival serving measurement")
    ap.add_argument("--no-drop-in", action="store_true", help="skip the prove_bin / bg_prove_dir load measurement")
    ap.add_argument("--msm-only", action="store_true",
                    help="time only the standalone G1 MSM 2^20 (a small, single-kernel-family profiling target)")
    ap.add_argument("--msm-log2n", type=int, default=20, choices=range(10, 21), metavar="10..20",
                    help="with --msm-only: the G1 MSM's size (profiling captures of a smaller case)")
    ap.add_argument("--pair-rounds", type=int, default=-1, choices=range(-1, 13), metavar="-1..12",
                    help="with --msm-only: force the batch-affine pair rounds (-1: the library's model)")
    ap.add_argument("--ntt-only", action="store_true",
                    help="time only the forward NTT of 2^20 Fr elements (a single-kernel profiling target)")
    ap.add_argument("--data-root", default=os.environ.get("BG_BENCH_DATA", "/tmp/bg_bench"))
    return ap.parse_args()


# ---------------------------------------------------------------- distributed plumbing
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def aggregate_ms_per_proof(times_ms_per_rank_max: float, world: int, steps: int) -> float:
    """whole-job ms/proof: the slowest rank's time over all proofs of all ranks"""
    return times_ms_per_rank_max / (world * steps)


# ---------------------------------------------------------------- workload
def instance_dir(args) -> str:
    return os.path.join(args.data_root, "sq%d_s%d" % (args.log2n, args.seed))


def ensure_instance(args, dist: Dist, generator) -> str:
    path = instance_dir(args)
    marker = os.path.join(path, "COMPLETE")
    if dist.rank == 0 and not (os.path.exists(marker) and os.path.exists(os.path.join(path, "vk.bin"))):
        os.makedirs(path, exist_ok=True)
        generator(args.log2n, args.seed, path)
        open(marker, "w").write("ok\n")
    dist.barrier()
    return path


def window_counts(L, n):
    c = L.bg_msm_window_bits(n, 0)
    return c, 254 // c + 1


def table_window_counts(L, n, curve=0):
    c = L.bg_msm_table_window_bits(n, curve)
    return c, 254 // c + 1


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region"""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        rows = [[c.strip() for c in ln.split(",")] for ln in out.splitlines() if ln.strip()]
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = set()
        for r in rows:
            for i, nm in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ---------------------------------------------------------------- our arm
def run_ours(args, dist: Dist):
    import numpy as np
    import torch

    import bendg
    torch.cuda.set_device(dist.local)
    ctx = bendg.Context(dist.local)
    L = bendg.lib()
    if args.ntt_only:
        # seeded Fr elements below 2^252 (< r), Montgomery form irrelevant to the transform's cost
        g = torch.Generator(device="cpu").manual_seed(args.seed)
        x = torch.randint(0, 1 << 30, ((1 << 20) * 8,), dtype=torch.int32, generator=g).cuda()
        x.view(-1, 8)[:, 7] &= 0x0FFFFFFF
        ext = torch.cuda.ExternalStream(ctx.stream)
        out = []
        for i in range(max(3, args.warmup) + args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            ctx.ntt_dev(x.data_ptr(), 20, 0)
            e1.record(ext)
            e1.synchronize()
            if i >= max(3, args.warmup):
                out.append(e0.elapsed_time(e1))
        ms = statistics.median(out)
        ops, pms = ctx.probe_imad(0, 4096)
        ctx.close()
        return {"metric": "NTT 2^20 forward ms", "value": round(ms, 4), "unit": "ms", "higher_is_better": False,
                "roofline": ntt_roofline(20, round(ms, 4), ops / (pms * 1e-3))}
    path = ensure_instance(args, dist, lambda k, s, p: ctx.synth_square_chain(k, s, p))
    files = bendg.HostFiles(path, pinned=True)
    hdr = files.words("header")
    nc, ni, nw, lg, na, nb, nh, nl = (int(v) for v in hdr[:8])

    if args.msm_only:
        import torch
        flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
        ext = torch.cuda.ExternalStream(ctx.stream)
        ops, ms = ctx.probe_imad(0, 4096)
        ctx.pair_rounds_override(args.pair_rounds)
        prims = primitives(ctx, files, nh, nb, args, ext, flush, ops / (ms * 1e-3), only_g1=True)
        ctx.close()
        key = "g1_msm_2^%d_ms" % args.msm_log2n
        return {"metric": "G1 MSM 2^%d ms" % args.msm_log2n, "value": prims[key], "unit": "ms",
                "higher_is_better": False, "pair_rounds": prims["pair_rounds"], "roofline": prims["roofline"]}

    # resident proving key + device witness (inputs in HBM before the timed region)
    key = ctx.pk_upload(files)
    wit = torch.from_numpy(files.words("witness").astype(np.int64).astype(np.int32)).cuda()
    rs = files.words("rs").copy()
    rs_ptr = rs.ctypes.data
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    ext = torch.cuda.ExternalStream(ctx.stream)

    def step_resident():
        return key.prove_ptr(wit.data_ptr(), rs_ptr)

    for _ in range(max(3, args.warmup)):
        step_resident()
    # IMAD peak of this GPU, measured before the timed region
    ops, ms = ctx.probe_imad(0, 4096)
    imad_peak = ops / (ms * 1e-3)
    ops_f, ms_f = ctx.probe_imad(1, 256)
    fqmul_rate = ops_f / (ms_f * 1e-3)

    launches0 = ctx.launches()
    clocks = ClockSampler(dist.local)
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    step_ms, phases = [], []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        last_proof, t = step_resident()
        e1.record(ext)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        phases.append(t)
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    # the last timed proof must pass the pairing verifier under the instance's verifying key
    vkw = np.fromfile(os.path.join(path, "vk.bin"), dtype="<u4").astype(np.uint32)
    n_ic = int(vkw[224])
    verified = bendg.verify(vkw[0:32], vkw[32:96], vkw[96:160], vkw[160:224], vkw[225:225 + 32 * n_ic],
                            files.words("witness")[16:16 * n_ic], last_proof)
    launches = ctx.launches() - launches0
    total = dist.max(sum(step_ms))
    value = aggregate_ms_per_proof(total, dist.world, args.steps)

    # per-kernel times from an untimed pass of the same proofs with the library's kernel timers
    # on (events around every launch), so that the timed proofs above run without them
    ctx.profile(True)
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        step_resident()
    torch.cuda.synchronize()
    # roofline of the dominant kernel (the one with the largest summed time)
    fams = KERNEL_FAMILIES
    stats = {f: ctx.kernel_stats(f) for f in fams}
    ctx.profile(False)
    dom = "msm_bucket_acc_g1"
    g1_sizes = [na, nb, nh, nl]
    # the timed proofs run against the resident key: window tables, W = floor(254 / c_table) + 1
    entries_g1 = sum(n * table_window_counts(L, n)[1] for n in g1_sizes)
    entries_g2 = nb * table_window_counts(L, nb, 1)[1]
    work = {"msm_bucket_acc_g1": entries_g1 * MADD_G1_IMAD,
            "msm_bucket_acc_g2": entries_g2 * MADD_G2_IMAD}
    roof = None
    if dom in work:
        nl_, tms = stats[dom]
        per_launch_work = work[dom] * args.steps / max(1, nl_)
        avg_ms = tms / max(1, nl_)
        achieved = per_launch_work / (avg_ms * 1e-3) / 1e9
        traffic, traffic_src = traffic_record(dom)
        roof = {"kernel": dom, "traffic_source": traffic_src,
                "where": "inside the proof (a profiled pass of the timed proofs): avg_launch_ms is the event span "
                         "around each launch on its stream while 4 other streams run concurrently, so it is an "
                         "upper bound of the kernel's own duration and frac a lower bound",
                "bound": "imad", "achieved": round(achieved, 1), "peak": round(imad_peak / 1e9, 1),
                "unit": "Gimad/s", "frac": round(achieved / (imad_peak / 1e9), 4), "traffic": traffic,
                "work_per_launch": per_launch_work, "avg_launch_ms": round(avg_ms, 4),
                "peak_source": "bg_probe_imad on this GPU (32-bit mad.lo/mad.hi chains)",
                "work_model": "entries x %d IMAD per G1 mixed add (G2: %d)" % (MADD_G1_IMAD, MADD_G2_IMAD)}
    kernel_ms = {f: {"launches": v[0], "ms_per_proof": round(v[1] / args.steps, 3)} for f, v in stats.items()}

    # e2e: all .bin files from pinned host memory through bg_prove_host, every step (after the
    # same number of warm-up calls as the resident-key steps)
    for _ in range(max(3, args.warmup)):
        ctx.prove_host(files)
    dist.barrier()
    torch.cuda.synchronize()
    e2e_ms = []
    xfer0 = ctx.transfer_bytes()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        ctx.prove_host(files)
        e1.record(ext)
        e1.synchronize()
        e2e_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    xfer1 = ctx.transfer_bytes()
    dist.barrier()
    e2e_total = dist.max(sum(e2e_ms))
    # bytes the library copied (its own counters: file uploads, MSM window sums, status words)
    e2e = {"value": round(aggregate_ms_per_proof(e2e_total, dist.world, args.steps), 3), "unit": UNIT,
           "h2d_bytes_per_step": (xfer1[0] - xfer0[0]) // args.steps,
           "d2h_bytes_per_step": (xfer1[1] - xfer0[1]) // args.steps,
           "api": "bg_prove_host (every .bin file uploaded per proof)",
           "step_ms_min": round(min(e2e_ms), 3), "step_ms_median": round(statistics.median(e2e_ms), 3),
           "steps_ms": [round(t, 2) for t in e2e_ms]}
    # Split of e2e - value: the same one-shot call with the five query sets (pk_a .. pk_l, all
    # but 8 MB of the files) already in device memory, which bg_prove_host then copies device to
    # device, isolates the host-to-device transfer from the one-shot MSM layout (a bucket set per
    # window, no window tables) that the resident key's tables avoid
    dev_sets = {nm: torch.from_numpy(files.bufs[nm].view(np.int32)).cuda()
                for nm in ("pk_a", "pk_b1", "pk_b2", "pk_h", "pk_l")}
    import bendg as _b
    dev_in = _b.Inputs.from_buffer_copy(files.inputs)
    for nm, t in dev_sets.items():
        setattr(dev_in, nm, t.data_ptr())
    torch.cuda.synchronize()
    for _ in range(2):
        ctx.prove_inputs(dev_in)
    sets_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        ctx.prove_inputs(dev_in)
        e1.record(ext)
        e1.synchronize()
        sets_ms.append(e0.elapsed_time(e1))
    on_dev = statistics.median(sets_ms)
    e2e["split"] = {"query_sets_in_device_memory_ms": round(on_dev, 3),
                    "host_transfer_ms": round(e2e["value"] - on_dev, 3),
                    "one_shot_layout_ms": round(on_dev - value, 3),
                    "how": "e2e - (the same bg_prove_host call with the five query sets already on the device) "
                           "= transfer; that call - value (resident key with window tables) = layout"}
    del dev_sets

    prims = None if args.no_primitives else primitives(ctx, files, nh, nb, args, ext, flush, imad_peak)
    roof_iso = prims.pop("roofline") if prims else None
    batch = None if args.no_batch else batched(ctx, args, flush, ext, imad_peak)
    serve = None if args.no_serve else serving(ctx, args)
    dropin = None if args.no_drop_in else drop_in(ctx, args)

    result = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(value * dist.world, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": round(value / REF_GPU_K18_MS, 6),
        "vs_baseline_ref": "Bend 2 CUDA path, RTX 5090, K=18 T total 56083 ms (bend2/bench/prover_results.md:63)",
        "dtype": "u32 (exact BN254 Fr/Fq Montgomery arithmetic)", "data": "synthetic (seeded SquareChain instance)",
        "config": workload_config(args, lg, na, nb, nh, nl, dist.world),
        "msm": {"window_bits": {"g1": {str(n): L.bg_msm_table_window_bits(n, 0) for n in sorted(set(g1_sizes))},
                                "g2": {str(nb): L.bg_msm_table_window_bits(nb, 1)}},
                "layout": "resident key: 2^(c w) window tables, one shared bucket set per MSM"},
        "proof_verified": bool(verified),
        "e2e": e2e, "roofline": roof_iso or roof, "roofline_in_proof": roof, "gpu_launches": int(launches), "clocks": clk,
        "phases_ms_median": {k: round(statistics.median(p[k] for p in phases), 3) for k in phases[0]},
        "kernels": kernel_ms, "fq_mul_rate_gops": round(fqmul_rate / 1e9, 2), "primitives": prims,
        "batched": batch, "serving": serve, "drop_in": dropin,
    }
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(path, samples=3)
    key.release()
    files.free()
    ctx.close()
    return result


BATCH_KS = (10, 12, 14, 16, 18)
BATCH_WEIGHTS = (0.3, 0.25, 0.2, 0.15, 0.1)
P_FR = 21888242871839275222246405745257275088548364400416034343698204186575808495617


def shifted_witness(z_words, m: int):
    """SquareChain witness for x0' = x_m, built from the instance witness
    z = [1, x_N, x_0 .. x_{N-1}] (Montgomery wire words) and m more squarings of x_N:
    z' = [1, x_{N+m}, x_m .. x_{N-1}, x_N .. x_{N+m-1}]"""
    import numpy as np
    import bendg
    w = np.asarray(z_words, dtype=np.uint32).reshape(-1, 16)
    r_inv = pow(1 << 256, -1, P_FR)
    xn = bendg.wire_to_ints(w[1])[0] * r_inv % P_FR
    ext = []
    x = xn
    for _ in range(m):
        x = x * x % P_FR
        ext.append(x)  # x_{N+1} .. x_{N+m}
    mont = [v * (1 << 256) % P_FR for v in [xn] + ext]
    tail = bendg.ints_to_wire(mont[:m])            # x_N .. x_{N+m-1}
    head = bendg.ints_to_wire([mont[m]])           # x_{N+m}
    return np.concatenate([w[0:1], head, w[2 + m:], tail]).reshape(-1)


def proof_imad(L, hdr) -> int:
    """algorithmic 32-bit multiply-adds of one resident-key proof: every MSM entry one mixed
    addition (n W per MSM with W the window-table rows: G1 2136, G2 5136 IMAD) and the 7 NTTs of
    the QAP ((d / 2) log2 d Fr products of 232 IMAD); the window reductions are left out, so a
    fraction of the probed peak computed from it is a lower bound"""
    nc, ni, nw, lg, na, nb, nh, nl = (int(v) for v in hdr[:8])
    g1 = sum(n * table_window_counts(L, n)[1] for n in (na, nb, nh, nl) if n)
    g2 = nb * table_window_counts(L, nb, 1)[1]
    d = 1 << lg
    return g1 * MADD_G1_IMAD + g2 * MADD_G2_IMAD + 7 * (d // 2) * lg * 232


def batched(ctx, args, flush, ext, imad_peak=None):
    """The batch workload: 64 proofs of mixed K, one bg_prove_batch call versus the same
    proofs made one at a time (plain), both against resident keys; every batched proof must
    equal its plain twin bit for bit."""
    import random

    import numpy as np
    import torch

    import bendg
    rng = random.Random(args.seed + 3)
    keys, wits = {}, {}
    files = {}
    for k in BATCH_KS:
        a = argparse.Namespace(**vars(args))
        a.log2n = k
        single = Dist.__new__(Dist)
        single.world, single.rank, single.local, single.pg = 1, 0, 0, None
        path = ensure_instance(a, single, lambda kk, s, p: ctx.synth_square_chain(kk, s, p))
        files[k] = bendg.HostFiles(path)
        keys[k] = ctx.pk_upload(files[k])
        wits[k] = files[k].words("witness").copy()
    ks = rng.choices(BATCH_KS, weights=BATCH_WEIGHTS, k=64)
    jobs = []
    for i, k in enumerate(ks):
        w = shifted_witness(wits[k], 1 + i)
        r, s = rng.randrange(P_FR), rng.randrange(P_FR)
        rs = bendg.ints_to_wire([r * (1 << 256) % P_FR, s * (1 << 256) % P_FR]).reshape(-1)
        jobs.append((k, w, rs))

    def plain():
        return [keys[k].prove(w, rs)[0] for k, w, rs in jobs]

    def batch(lanes):
        proofs, _, st = ctx.prove_batch([keys[k] for k, _, _ in jobs], [w for _, w, _ in jobs],
                                        [rs for _, _, rs in jobs], lanes=lanes)
        assert all(s == bendg.BG_OK for s in st)
        return proofs

    def timed(fn):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        out = fn()
        e1.record(ext)
        e1.synchronize()
        return out, e0.elapsed_time(e1)

    plain(), batch(8)  # warm every lane and workspace
    ref, t_plain = timed(plain)
    lanes_best, t_best, got = None, None, None
    for lanes in BATCH_LANES:
        out, t = timed(lambda: batch(lanes))
        if t_best is None or t < t_best:
            lanes_best, t_best, got = lanes, t, out
    exact = all(ctx.proof_text(a) == ctx.proof_text(b) for a, b in zip(got, ref))
    for k in BATCH_KS:
        keys[k].release()
    # the batch against the multiply-add roofline: its algorithmic IMAD over the batched time and
    # the probed rate; batched >= 2x plain would need the plain fraction doubled
    L = bendg.lib()
    work = sum(proof_imad(L, files[k].words("header")) for k in ks)
    roof = None
    if imad_peak:
        roof = {"work_imad": work, "peak_gimad_s": round(imad_peak / 1e9, 1),
                "batched_frac": round(work / (t_best * 1e-3) / imad_peak, 4),
                "plain_frac": round(work / (t_plain * 1e-3) / imad_peak, 4),
                "frac_needed_for_2x_plain": round(2 * work / (t_plain * 1e-3) / imad_peak, 4),
                "model": "per proof: MSM entries (n W with the window-table W) x 2136 (G1) / 5136 (G2) IMAD + "
                         "7 NTTs x (d/2) log2 d x 232; reductions left out (a lower bound)",
                "best_kernel_frac_alone": "the XYZZ accumulation reaches 0.76 of the probe running alone "
                                          "(G1 MSM 2^20, one bucket set per window)"}
    return {"workload": "64 SquareChain proofs, K drawn from %s with weights %s (seed %d), resident keys"
                        % (list(BATCH_KS), list(BATCH_WEIGHTS), args.seed + 3),
            "k_counts": {str(k): ks.count(k) for k in BATCH_KS},
            "plain_ms": round(t_plain, 2), "plain_proofs_per_s": round(64 / (t_plain * 1e-3), 1),
            "batched_ms": round(t_best, 2), "batched_proofs_per_s": round(64 / (t_best * 1e-3), 1),
            "speedup_vs_plain": round(t_plain / t_best, 3), "lanes": lanes_best,
            "bit_exact_vs_plain": bool(exact), "roofline": roof}


# lanes (concurrent provers) the batch is timed with (the best is reported)
BATCH_LANES = (4, 8, 12)
SERVE_KS = (12, 14, 16, 18, 20)
SERVE_LANES = 8
SERVE_HBM_BUDGET = 64 << 30
SERVE_WEIGHTS = (0.3, 0.25, 0.2, 0.15, 0.1)
SERVE_RATES = (10, 50, 100, 200, 500)


def percentile(xs, q):
    s = sorted(xs)
    if not s:
        return None
    i = min(len(s) - 1, max(0, int(round(q / 100.0 * (len(s) - 1)))))
    return s[i]


def single_proofs(ctx, key, path, reps=5):
    """The single-proof workload at its larger size (2^20 constraints): plain one-at-a-time
    proofs against a resident key (wall time of the synchronous call, device work included),
    and the pairing check of the last one under the instance's vk.bin"""
    import numpy as np

    import bendg
    f = bendg.HostFiles(path, pinned=True)
    w, rs = f.words("witness"), f.words("rs")
    for _ in range(2):
        key.prove(w, rs)
    walls, phases = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        proof, t = key.prove(w, rs)
        walls.append((time.perf_counter() - t0) * 1e3)
        phases.append(t)
    vkw = np.fromfile(os.path.join(path, "vk.bin"), dtype="<u4").astype(np.uint32)
    n_ic = int(vkw[224])
    ok = bendg.verify(vkw[0:32], vkw[32:96], vkw[96:160], vkw[160:224], vkw[225:225 + 32 * n_ic],
                      w[16:16 * n_ic], proof)
    hdr = f.words("header")
    return {"log2_constraints": int(hdr[0]).bit_length() - 1, "ms_per_proof": round(statistics.median(walls), 3),
            "phases_ms_median": {k: round(statistics.median(p[k] for p in phases), 3) for k in phases[0]},
            "proof_verified": bool(ok), "timing": "wall clock of bg_prove_resident, median of %d" % reps}


def serving(ctx, args, lanes=None, seconds=1.5, budget=None):
    """The serving workload: Poisson arrivals of prove requests with K drawn from
    SERVE_KS, all five proving keys resident, continuous batching in the library's server;
    p50 / p99 latency (submit -> proof) and completed proofs/s per offered rate."""
    import random
    import threading

    import bendg
    rng = random.Random(args.seed + 4)
    keys, pools, paths = {}, {}, {}
    for k in SERVE_KS:
        a = argparse.Namespace(**vars(args))
        a.log2n = k
        single = Dist.__new__(Dist)
        single.world, single.rank, single.local, single.pg = 1, 0, 0, None
        path = ensure_instance(a, single, lambda kk, s, p: ctx.synth_square_chain(kk, s, p))
        f = bendg.HostFiles(path)
        keys[k] = ctx.pk_upload(f)
        z = f.words("witness").copy()
        pools[k] = [shifted_witness(z, 1 + j) for j in range(4)]  # distinct valid witnesses
        paths[k] = path
        del f
    k20 = single_proofs(ctx, keys[SERVE_KS[-1]], paths[SERVE_KS[-1]])
    lanes = lanes or SERVE_LANES
    budget = budget or SERVE_HBM_BUDGET
    srv = bendg.Server(ctx, lanes=lanes, hbm_budget_bytes=budget)
    # warm every lane on the largest key
    for t in range(lanes):
        srv.submit(keys[SERVE_KS[-1]], pools[SERVE_KS[-1]][0], bendg.ints_to_wire([1, 1]).reshape(-1), 10**9 + t)
    for _ in range(lanes):
        srv.wait(600000)
    results = []
    served, all_reqs = {}, []
    tag = 0
    for rate in SERVE_RATES:
        n = max(12, int(rate * seconds))
        arrivals, t = [], 0.0
        for _ in range(n):
            t += rng.expovariate(rate)
            arrivals.append(t)
        reqs = []
        for _ in range(n):
            k = rng.choices(SERVE_KS, weights=SERVE_WEIGHTS, k=1)[0]
            rs = bendg.ints_to_wire([rng.randrange(P_FR) * (1 << 256) % P_FR,
                                     rng.randrange(P_FR) * (1 << 256) % P_FR]).reshape(-1)
            reqs.append((tag, k, rng.choice(pools[k]), rs))
            tag += 1
        lat, done_at = {}, []

        def collect():
            while len(lat) < n:
                r = srv.wait(600000)
                if r is None:
                    return
                assert r[5] == bendg.BG_OK
                lat[r[0]] = r[3]
                served[r[0]] = bytes(r[1])
                done_at.append(time.perf_counter())

        th = threading.Thread(target=collect)
        th.start()
        t0 = time.perf_counter()
        for (tg, k, w, rs), at in zip(reqs, arrivals):
            now = time.perf_counter() - t0
            if at > now:
                time.sleep(at - now)
            srv.submit(keys[k], w, rs, tg)
        th.join()
        span = max(done_at) - t0
        all_reqs.extend(reqs)
        vals = list(lat.values())
        results.append({"offered_rps": rate, "requests": n, "completed": len(vals),
                        "p50_ms": round(percentile(vals, 50), 2), "p99_ms": round(percentile(vals, 99), 2),
                        "mean_ms": round(sum(vals) / len(vals), 2), "proofs_per_s": round(len(vals) / span, 1),
                        "k_counts": {str(k): sum(1 for r in reqs if r[1] == k) for k in SERVE_KS}})
    reserved = srv.reserved_bytes()
    srv.close()
    # After the timed windows: every served proof against the same request proved alone on the
    # plain path (bit for bit), and the pairing check of one served proof per K under its vk.bin
    import numpy as np
    mismatch = {str(r["offered_rps"]): 0 for r in results}
    rate_of = {}
    base = 0
    for r in results:
        for t in range(base, base + r["requests"]):
            rate_of[t] = str(r["offered_rps"])
        base += r["requests"]
    verified = {}
    for tg, k, w, rs in all_reqs:
        alone, _ = keys[k].prove(w, rs)
        if bytes(alone) != served.get(tg):
            mismatch[rate_of[tg]] += 1
        if str(k) not in verified:
            vkw = np.fromfile(os.path.join(paths[k], "vk.bin"), dtype="<u4").astype(np.uint32)
            n_ic = int(vkw[224])
            verified[str(k)] = bool(bendg.verify(vkw[0:32], vkw[32:96], vkw[96:160], vkw[160:224],
                                                 vkw[225:225 + 32 * n_ic], w[16:16 * n_ic], alone))
    for r in results:
        r["bit_exact_vs_alone"] = mismatch[str(r["offered_rps"])] == 0
    for k in SERVE_KS:
        keys[k].release()
    return {"workload": "Poisson arrivals, K drawn from %s with weights %s (seed %d), %s s of arrivals per rate, "
                        "all five keys resident" % (list(SERVE_KS), list(SERVE_WEIGHTS), args.seed + 4, seconds),
            "lanes": lanes, "hbm_budget_bytes": budget, "reserved_scratch_bytes": reserved, "rates": results,
            "bit_exact_vs_alone": all(v == 0 for v in mismatch.values()) and len(served) == len(all_reqs),
            "served_proofs_checked": len(all_reqs),
            "exactness_check": "after the timed windows, every served proof compared word for word with the "
                               "same (key, witness, r, s) proved alone by bg_prove_resident",
            "verified_per_k": verified, "single_proof_k20": k20}


def drop_in(ctx, args, ks=(18, 20), reps=3):
    """The drop-in path of bend2/scripts/prove.sh: the prove_bin CLI (a new process per proof,
    BENDG_DATA pointing at the instance's .bin files, warm page cache) and bg_prove_dir in a warm
    process, with the T lines the library reports; the reference's T load for the same sizes is
    883 ms (K=18) and 3,502 ms (K=20) (bend2/bench/prover_results.md:59, :60)"""
    out = {}
    binp = os.path.join(PKG, "prove_bin")
    for k in ks:
        a = argparse.Namespace(**vars(args))
        a.log2n = k
        single = Dist.__new__(Dist)
        single.world, single.rank, single.local, single.pg = 1, 0, 0, None
        path = ensure_instance(a, single, lambda kk, s, p: ctx.synth_square_chain(kk, s, p))
        nbytes = sum(os.path.getsize(os.path.join(path, f)) for f in os.listdir(path) if f.endswith(".bin"))
        env = dict(os.environ, BENDG_DATA=path)
        cli = []
        for rep in range(reps + 1):  # the first run warms the page cache
            t0 = time.perf_counter()
            r = subprocess.run([binp], env=env, capture_output=True, text=True, check=True)
            wall = (time.perf_counter() - t0) * 1e3
            T = {ln.split()[1]: float(ln.split()[2]) for ln in r.stdout.splitlines() if ln.startswith("T ")}
            if rep:
                cli.append((wall, T, "".join(ln + "\n" for ln in r.stdout.splitlines() if ln[:2] in ("A ", "B ", "C "))))
        inproc = []
        for _ in range(reps + 1):
            proof, t = ctx.prove_dir(path)
            inproc.append(t)
        inproc = inproc[1:]
        med = statistics.median
        out["k%d" % k] = {
            "bytes_read": nbytes,
            "cli_wall_ms": round(med(c[0] for c in cli), 1),
            "cli_T_load_ms": med(c[1]["load"] for c in cli), "cli_T_total_ms": med(c[1]["total"] for c in cli),
            "in_process_T_load_ms": round(med(t["load"] for t in inproc), 2),
            "in_process_T_total_ms": round(med(t["total"] for t in inproc), 2),
            "same_proof_cli_and_in_process": all(c[2] == ctx.proof_text(proof) for c in cli),
            "reference_T_load_ms": {18: 883, 20: 3502}.get(k)}
    return out


def primitives(ctx, files, nh, nb, args, ext, flush, imad_peak, only_g1=False):
    """the standalone primitives: G1 MSM 2^20, G2 MSM 2^18,
    NTT 2^20, all device-resident (points: the instance's h_query twice, as the reference's own
    MSM bench does for 2^20, bend2/bench/msm.bend:1-9; scalars uniform < r)"""
    import numpy as np
    import torch
    dev = torch.device("cuda")
    rng = np.random.default_rng(args.seed)

    def scalars(n):
        # uniform below 0x30644e72 * 2^224 < r (all but 2^-33 of [0, r)): every window of the
        # digit expansion, the top one included, sees the spread of a real witness
        w = rng.integers(0, 1 << 32, size=(n, 8), dtype=np.uint64).astype(np.uint32)
        w[:, 7] = rng.integers(0, 0x30644e72, size=n, dtype=np.uint64).astype(np.uint32)
        return torch.from_numpy(w.view(np.int32)).to(dev)

    def packed(name, count_words16):
        w = files.words(name)[:count_words16].astype(np.int64).astype(np.int32)
        d_wire = torch.from_numpy(w).to(dev)
        d_pk = torch.empty(count_words16 // 2, dtype=torch.int32, device=dev)
        ctx.repack_to_packed_dev(d_wire.data_ptr(), d_pk.data_ptr(), count_words16 // 16)
        torch.cuda.synchronize()
        return d_pk

    def timeit(fn, reps=5):
        for _ in range(2):
            fn()
        out = []
        for _ in range(reps):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            fn()
            e1.record(ext)
            e1.synchronize()
            out.append(e0.elapsed_time(e1))
        return round(statistics.median(out), 3)

    res = {}
    lg1 = args.msm_log2n if only_g1 else 20
    n1 = 1 << lg1
    h = packed("pk_h", nh * 32)
    a = packed("pk_a", 2 * 32)
    pts = torch.cat([h, h, a])[: n1 * 16].contiguous()
    sc = scalars(n1)
    res["g1_msm_2^%d_ms" % lg1] = timeit(lambda: ctx.msm_g1_dev(pts.data_ptr(), sc.data_ptr(), n1))
    # roofline of the MSM's dominant kernel running alone (events around each launch): the
    # batch-affine pair rounds when the library takes them for this size, else the XYZZ
    # accumulation; work counted exactly from these scalars' bucket sizes
    import bendg
    L = bendg.lib()
    ctx.profile(True)
    reps = 3
    for _ in range(reps):
        ctx.msm_g1_dev(pts.data_ptr(), sc.data_ptr(), n1)
    stats = {f: ctx.kernel_stats(f) for f in ("msm_pair_g1", "msm_bucket_acc_g1")}
    ctx.profile(False)
    c, W = window_counts(L, n1)
    rounds = L.bg_msm_pair_rounds(n1, 0) if args.pair_rounds < 0 or not only_g1 else args.pair_rounds
    res["pair_rounds"] = rounds
    counts = bucket_counts(sc.cpu().numpy().view(np.uint32).reshape(n1, 8), c)
    pair_adds = pair_round_additions(counts, rounds)
    if rounds:
        kern, work = "msm_pair_g1", sum(pair_adds) * PAIR_G1_IMAD
        model = ("%d batch-affine rounds: %s affine additions x %d IMAD (5 products + 1 square: 3 for the "
                 "shared inversion, the slope, its square and y3), counted from the scalars' bucket sizes "
                 "(c=%d, W=%d, %d entries)" % (rounds, "+".join(str(a) for a in pair_adds), PAIR_G1_IMAD, c, W,
                                               int(counts.sum())))
        where = "G1 MSM 2^%d alone: k_pair_round, %d launches per MSM timed as one span" % (lg1, rounds)
    else:
        kern, work = "msm_bucket_acc_g1", int(counts.sum()) * MADD_G1_IMAD
        model = "%d entries x %d IMAD per mixed add (c=%d, W=%d)" % (int(counts.sum()), MADD_G1_IMAD, c, W)
        where = "G1 MSM 2^%d alone" % lg1
    launches, tms = stats[kern]
    avg = tms / max(1, launches)
    achieved = work / (avg * 1e-3) / 1e9
    traffic, traffic_src = traffic_record("%s_2^%d" % (kern, lg1))
    res["roofline"] = {"kernel": kern, "where": where, "traffic_source": traffic_src,
                       "bound": "imad", "achieved": round(achieved, 1), "peak": round(imad_peak / 1e9, 1),
                       "unit": "Gimad/s", "frac": round(achieved / (imad_peak / 1e9), 4), "traffic": traffic,
                       "work_per_launch": work, "avg_launch_ms": round(avg, 4), "launches": launches,
                       "peak_source": "bg_probe_imad on this GPU (32-bit mad.lo/mad.hi chains)",
                       "work_model": model,
                       "accumulation_after_rounds_ms": round(stats["msm_bucket_acc_g1"][1] /
                                                             max(1, stats["msm_bucket_acc_g1"][0]), 4),
                       "hbm": acc_hbm_view(n1, c, W, avg, traffic)}
    if only_g1:
        return res
    n2 = 1 << 18
    b2 = packed("pk_b2", nb * 64)[: n2 * 32].contiguous()
    sc2 = scalars(n2)
    res["g2_msm_2^18_ms"] = timeit(lambda: ctx.msm_g2_dev(b2.data_ptr(), sc2.data_ptr(), n2))
    x = scalars(n1)
    res["ntt_2^20_forward_ms"] = timeit(lambda: ctx.ntt_dev(x.data_ptr(), 20, 0) or torch.cuda.synchronize())
    res["coset_ntt_2^20_ms"] = timeit(lambda: ctx.ntt_dev(x.data_ptr(), 20, 2) or torch.cuda.synchronize())
    res["ntt_roofline"] = ntt_roofline(20, res["ntt_2^20_forward_ms"], imad_peak)
    return res


def acc_hbm_view(n, c, W, avg_ms, traffic=None):
    """the G1 accumulation kernel against the HBM roofline: its minimal bytes per launch are
    the n affine points read once (64 B each), the n W entry codes read (4 B each) and the W
    2^(c-1) XYZZ buckets written (128 B each); the slice pieces of cut buckets come on top, so
    this is a lower bound.  The kernel is bound by its multiply-adds, so the fraction is small."""
    hbm_gbs = None
    pf = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pf):
        hbm_gbs = json.load(open(pf)).get("hbm_gbs")
    min_bytes = n * 64 + n * W * 4 + W * (1 << (c - 1)) * 128
    achieved = min_bytes / (avg_ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_gbs, "unit": "GB/s",
            "frac": round(achieved / hbm_gbs, 4) if hbm_gbs else None, "traffic": traffic,
            "algorithmic_bytes": min_bytes,
            "model": "points n x 64 B + entry codes n W x 4 B + buckets W 2^(c-1) x 128 B (lower bound)",
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}


def ntt_roofline(lg, ms, imad_peak):
    """both bounds of a forward NTT of 2^lg Fr elements: HBM (each element read and written
    once, 2 x 32 B) against the measured copy bandwidth, and the multiply-adds of its
    butterflies ((n/2) log2 n Fr products of 232: a 512-bit Karatsuba product and one
    Montgomery reduction) against the probed IMAD rate; the larger time is the binding bound"""
    n = 1 << lg
    hbm_gbs = None
    pf = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pf):
        hbm_gbs = json.load(open(pf)).get("hbm_gbs")
    min_bytes = 2 * 32 * n
    work = (n // 2) * lg * 232
    t_imad = work / imad_peak * 1e3
    t_hbm = min_bytes / (hbm_gbs * 1e9) * 1e3 if hbm_gbs else None
    bound = "imad" if t_hbm is None or t_imad >= t_hbm else "hbm"
    return {"n": n, "ms": ms, "bound": bound,
            "imad": {"work": work, "bound_ms": round(t_imad, 4), "achieved_gimad_s": round(work / (ms * 1e-3) / 1e9, 1),
                     "frac": round(t_imad / ms, 4), "peak_source": "bg_probe_imad"},
            "hbm": {"min_bytes": min_bytes, "bound_ms": round(t_hbm, 4) if t_hbm else None,
                    "moved_bytes_2_pass_plan": 2 * min_bytes,
                    "achieved_gbs": round(2 * min_bytes / (ms * 1e-3) / 1e9, 1),
                    "frac": round(t_hbm / ms, 4) if t_hbm else None,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}}


# ---------------------------------------------------------------- CPU restatement
def traffic_record(key: str):
    """DRAM bytes per launch of a kernel from the committed ncu summary (profiles/
    roofline_traffic.json), with the capture's date, commit and command: ncu cannot run inside
    the timed bench, so the figure is as current as that capture"""
    tf = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if not os.path.exists(tf):
        return None, None
    e = json.load(open(tf)).get(key)
    if not e:
        return None, None
    return e.get("bytes_per_launch"), "%s (captured %s at commit %s)" % (e.get("source"), e.get("captured", "?"),
                                                                       e.get("commit", "?"))


def workload_config(args, lg, na, nb, nh, nl, world):
    """the `config` both arms print: the same keys and values for the same workload"""
    return {"workload": "SquareChain(2^%d) Groth16 proof: 4 G1 MSMs + 1 G2 MSM + 7 radix-2 NTTs of 2^%d"
                        % (args.log2n, lg),
            "log2_constraints": args.log2n, "domain_log2": lg, "n_a": na, "n_b": nb, "n_h": nh, "n_l": nl,
            "seed": args.seed, "parallelism": "replicas" if world > 1 else "single device",
            "l2": "inputs larger than L2 (proving key and witness, 308 MB at 2^18); the GPU arm also flushes L2 "
                  "(512 MiB write) before every timed step"}


def cpu_baseline(path: str, samples: int = 3) -> dict:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_c
    threads = os.cpu_count() or 1
    oracle_c.prove_dir(path, threads)  # warm (page cache, thread pool)
    t = []
    for _ in range(samples):
        t0 = time.perf_counter()
        oracle_c.prove_dir(path, threads)
        t.append((time.perf_counter() - t0) * 1e3)
    return {"value": round(statistics.median(t), 1), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d complete proof(s) of the same SquareChain instance (load, evals, qap, 5 MSMs, combine)"
                      % samples}


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ctypes

    import oracle_c
    L = oracle_c.lib()
    L.bgo_synth_square_chain.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_int]
    threads = os.cpu_count() or 1

    def gen(k, s, p):
        if L.bgo_synth_square_chain(k, s, p.encode(), threads) != 0:
            raise RuntimeError("oracle synth failed")

    single = Dist.__new__(Dist)
    single.world, single.rank, single.local, single.pg = 1, 0, 0, None
    path = ensure_instance(args, single, gen)
    for _ in range(args.warmup):
        oracle_c.prove_dir(path, threads)
    t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle_c.prove_dir(path, threads)
        t.append((time.perf_counter() - t0) * 1e3)
    value = sum(t) / len(t)
    hdr = open(os.path.join(path, "header.bin"), "rb").read()
    import struct
    nc, ni, nw, lg, na, nb, nh, nl = struct.unpack("<8I", hdr)
    return {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "impl": "reference", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(value, 1), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": round(value / REF_GPU_K18_MS, 6), "dtype": "u64 (exact BN254 arithmetic)",
        "data": "synthetic (seeded SquareChain instance)",
        "config": workload_config(args, lg, na, nb, nh, nl, dist.world),
        "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "one complete proof per step (the reference's Bend 2 / arkworks CPU provers "
                                   "cannot run on this image: C restatement in oracle/)"},
        "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    dist = Dist()
    try:
        res = run_reference(args, dist) if args.impl == "reference" else run_ours(args, dist)
        if res is not None and dist.rank == 0:
            print(json.dumps(res), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
