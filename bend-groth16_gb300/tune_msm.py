"""Window-width autotuner for the MSM: measures the fastest window width c per (log2 n, curve)
on the GPU it runs on and writes the table the library compiles in (csrc/msm_tune.h).

    python bend-groth16_gb300/tune_msm.py --out bend-groth16_gb300/csrc/msm_tune.h

Two layouts are tuned, as the library uses them:
  * one bucket set per window (bg_msm_g1/g2, one-shot proofs): the standalone MSM over n
    points for c in [rule - 2, rule + 2], widened while the fastest c is on an edge;
  * window tables of resident keys (one shared bucket set): whole SquareChain(2^K) proofs
    against a key uploaded with the table width of one curve forced to c in [rule - 1, rule + 1],
    widened the same way (every G1 query of that proof has floor(log2 n) = K, and so does the
    G2 one), G1 first, then G2 with G1 at its best;
  * one bucket set per window inside a proof: whole one-shot SquareChain(2^K) proofs
    (bg_prove_host) with one curve's width forced to c in [current - 2, current + 2], widened
    the same way.
Timings are medians of wall-clock calls of the synchronous API (device work included).  Sizes
the run skips keep 0 in the table (the library's size rule applies there).
"""
import argparse
import os
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import bendg  # noqa: E402

MIN_LOG2, MAX_LOG2 = 10, 22


def median_ms(fn, reps):
    for _ in range(2):
        fn()
    out = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        out.append((time.perf_counter() - t0) * 1e3)
    return statistics.median(out)


def same_result(seen, key, result):
    """a width changes how a result is computed, never what it is: the first result for `key`
    is kept, and any later width that gives another one stops the tuning"""
    if key not in seen:
        seen[key] = result
    elif seen[key] != result:
        raise RuntimeError("tune_msm: %s gave a different result at another window width" % (key,))


def search(measure, lo, hi, c_min, c_max):
    """times of c in [lo, hi] (clamped to [c_min, c_max]), the range widened one step at a time
    while the fastest width sits on an edge of it"""
    lo, hi = max(c_min, lo), min(c_max, hi)
    times = {c: measure(c) for c in range(lo, hi + 1)}
    while True:
        best = min(times, key=times.get)
        if best == lo and lo > c_min:
            lo -= 1
            times[lo] = measure(lo)
        elif best == hi and hi < c_max:
            hi += 1
            times[hi] = measure(hi)
        else:
            return times


def tune_sets(ctx, torch, pts_g1, pts_g2, log2s_g1, log2s_g2, reps, log):
    """layout 0: standalone MSMs over device-resident points and uniform scalars below r"""
    dev = torch.device("cuda")
    rng = np.random.default_rng(12345)
    best = {0: {}, 1: {}}
    seen = {}
    for curve, log2s, pts in ((bendg.CURVE_G1, log2s_g1, pts_g1), (bendg.CURVE_G2, log2s_g2, pts_g2)):
        pw = 16 if curve == bendg.CURVE_G1 else 32
        for lg in log2s:
            n = 1 << lg
            w = rng.integers(0, 1 << 32, size=(n, 8), dtype=np.uint64).astype(np.uint32)
            w[:, 7] = rng.integers(0, 0x30644e72, size=n, dtype=np.uint64).astype(np.uint32)
            sc = torch.from_numpy(w.view(np.int32)).to(dev)
            reps_needed = (n * pw + pts.numel() - 1) // pts.numel()
            p = pts.repeat(reps_needed)[: n * pw].contiguous()
            rule = bendg.lib().bg_msm_window_bits(n, curve)
            f = ctx.msm_g1_dev if curve == bendg.CURVE_G1 else ctx.msm_g2_dev

            def measure(c):
                ctx.window_override(0, curve, c)
                same_result(seen, ("sets", curve, lg), f(p.data_ptr(), sc.data_ptr(), n).tobytes())
                return median_ms(lambda: f(p.data_ptr(), sc.data_ptr(), n), reps)
            times = search(measure, rule - 2, rule + 2, 3, 20)
            ctx.window_override(0, curve, 0)
            c_best = min(times, key=times.get)
            best[curve][lg] = c_best
            log("sets  %s 2^%d: %s -> c=%d" % ("g1" if curve == 0 else "g2", lg,
                                              " ".join("%d:%.3f" % kv for kv in sorted(times.items())), c_best))
    return best


def tune_tables(ctx, ks, data_root, reps, log):
    """layout 1: resident-key proofs with one curve's table width forced"""
    best = {0: {}, 1: {}}
    seen = {}
    for k in ks:
        path = os.path.join(data_root, "sq%d" % k)
        if not os.path.exists(os.path.join(path, "vk.bin")):
            ctx.synth_square_chain(k, 4242 + k, path)
        files = bendg.HostFiles(path, pinned=True)
        w, rs = files.words("witness"), files.words("rs")
        hdr = files.words("header")
        forced = {0: 0, 1: 0}
        for curve in (bendg.CURVE_G1, bendg.CURVE_G2):
            n = int(hdr[4]) if curve == bendg.CURVE_G1 else int(hdr[5])
            rule = bendg.lib().bg_msm_table_window_bits(n, curve)

            def measure(c):
                for cv in (0, 1):
                    ctx.window_override(1, cv, forced[cv] if cv != curve else c)
                key = ctx.pk_upload(files)
                same_result(seen, ("table", k), ctx.proof_text(key.prove(w, rs)[0]))
                t = median_ms(lambda: key.prove(w, rs), reps)
                key.release()
                return t
            times = search(measure, rule - 1, rule + 1, 6, 20)
            c_best = min(times, key=times.get)
            forced[curve] = c_best
            best[curve][k] = c_best
            log("table %s K=%d: %s -> c=%d" % ("g1" if curve == 0 else "g2", k,
                                              " ".join("%d:%.3f" % kv for kv in sorted(times.items())), c_best))
        for cv in (0, 1):
            ctx.window_override(1, cv, 0)
    return best


def committed_tables(path):
    """the kTuneSets / kTuneTables / kTuneProofSets rows of an existing header, as
    {curve: {log2 n: c}} (nonzero only)"""
    import re
    rows = re.findall(r"\{([0-9, ]+)\}", open(path).read())
    out = []
    for r in rows[:6]:
        vals = [int(x) for x in r.split(",")]
        out.append({MIN_LOG2 + i: v for i, v in enumerate(vals) if v})
    while len(out) < 6:
        out.append({})
    return {0: out[0], 1: out[1]}, {0: out[2], 1: out[3]}, {0: out[4], 1: out[5]}


def tune_proof_sets(ctx, ks, data_root, reps, log):
    """layout 2: whole one-shot proofs (every file uploaded, one bucket set per window) with one
    curve's width forced; every G1 MSM of a SquareChain(2^K) proof has floor(log2 n) = K, and so
    does the G2 one"""
    best = {0: {}, 1: {}}
    seen = {}
    for k in ks:
        path = os.path.join(data_root, "sq%d" % k)
        if not os.path.exists(os.path.join(path, "vk.bin")):
            ctx.synth_square_chain(k, 4242 + k, path)
        files = bendg.HostFiles(path, pinned=True)
        forced = {0: 0, 1: 0}
        for curve in (bendg.CURVE_G1, bendg.CURVE_G2):
            rule = bendg.lib().bg_msm_proof_window_bits(1 << k, curve)

            def measure(c):
                for cv in (0, 1):
                    ctx.window_override(0, cv, forced[cv] if cv != curve else c)
                same_result(seen, ("proof", k), ctx.proof_text(ctx.prove_host(files)[0]))
                return median_ms(lambda: ctx.prove_host(files), reps)
            times = search(measure, rule - 2, rule + 2, 3, 20)
            c_best = min(times, key=times.get)
            forced[curve] = c_best
            best[curve][k] = c_best
            log("proof %s K=%d: %s -> c=%d" % ("g1" if curve == 0 else "g2", k,
                                              " ".join("%d:%.3f" % kv for kv in sorted(times.items())), c_best))
        for cv in (0, 1):
            ctx.window_override(0, cv, 0)
    return best


def header_text(sets, tables, gpu, proof_sets=None):
    proof_sets = proof_sets or {0: {}, 1: {}}

    def row(d):
        return "{" + ", ".join(str(d.get(lg, 0)) for lg in range(MIN_LOG2, MAX_LOG2 + 1)) + "}"
    return """// Window widths of the MSM per (log2 n, curve), measured on %s by bend-groth16_gb300/tune_msm.py
// and committed; 0 = not measured, the size rule of msm_pick_c / msm_pick_c_table applies
// (msm_pick_c_proof: the bucket-set-per-window entry).
// Rows: [0] G1, [1] G2; columns: floor(log2 n) = kTuneMinLog2 .. kTuneMaxLog2.
#pragma once

namespace bg {

constexpr int kTuneMinLog2 = %d;
constexpr int kTuneMaxLog2 = %d;
// one bucket set per window (standalone MSMs)
constexpr signed char kTuneSets[2][kTuneMaxLog2 - kTuneMinLog2 + 1] = {
    %s,
    %s};
// window tables of resident keys (one shared bucket set)
constexpr signed char kTuneTables[2][kTuneMaxLog2 - kTuneMinLog2 + 1] = {
    %s,
    %s};
// one bucket set per window inside a proof (one-shot proofs): the MSMs share the GPU with
// each other's reductions and the QAP, which moves the best width from the standalone one
constexpr signed char kTuneProofSets[2][kTuneMaxLog2 - kTuneMinLog2 + 1] = {
    %s,
    %s};

}  // namespace bg
""" % (gpu, MIN_LOG2, MAX_LOG2, row(sets[0]), row(sets[1]), row(tables[0]), row(tables[1]),
       row(proof_sets[0]), row(proof_sets[1]))


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--out", default=os.path.join(HERE, "csrc", "msm_tune.h"))
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--data-root", default="/tmp/bg_tune")
    ap.add_argument("--max-sets-log2", type=int, default=22)
    ap.add_argument("--table-ks", default="10,12,14,16,18,20")
    ap.add_argument("--proof-ks", default="10,12,14,16,18,20",
                    help="K of the one-shot SquareChain(2^K) proofs that tune the in-proof widths")
    ap.add_argument("--keep", default=None,
                    help="an existing msm_tune.h whose entries are kept where this run measures nothing")
    args = ap.parse_args()
    import torch
    ctx = bendg.Context(0)
    log_lines = []

    def log(s):
        print(s, flush=True)
        log_lines.append(s)

    sets = {0: {}, 1: {}}
    if args.max_sets_log2 >= MIN_LOG2:
        # base points: the h and b2 queries of a SquareChain(2^20) instance, tiled as needed
        base = os.path.join(args.data_root, "sq20")
        if not os.path.exists(os.path.join(base, "vk.bin")):
            ctx.synth_square_chain(20, 4262, base)
        files = bendg.HostFiles(base)
        dev = torch.device("cuda")

        def packed(name, count):
            words = files.words(name)
            n = words.size // (32 if name != "pk_b2" else 64)
            n = min(n, count)
            wire = torch.from_numpy(words[: n * (32 if name != "pk_b2" else 64)].astype(np.int64).astype(np.int32))
            wire = wire.to(dev)
            out = torch.empty(wire.numel() // 2, dtype=torch.int32, device=dev)
            ctx.repack_to_packed_dev(wire.data_ptr(), out.data_ptr(), wire.numel() // 16)
            torch.cuda.synchronize()
            return out

        pts_g1 = packed("pk_h", 1 << 21)
        pts_g2 = packed("pk_b2", 1 << 20)
        sets = tune_sets(ctx, torch, pts_g1, pts_g2, range(MIN_LOG2, args.max_sets_log2 + 1),
                         range(MIN_LOG2, min(args.max_sets_log2, 20) + 1), args.reps, log)
    tables = tune_tables(ctx, [int(k) for k in args.table_ks.split(",") if k], args.data_root, args.reps, log)
    proof_sets = tune_proof_sets(ctx, [int(k) for k in args.proof_ks.split(",") if k], args.data_root, args.reps,
                                 log)
    if args.keep:
        old_sets, old_tables, old_proof = committed_tables(args.keep)
        for new, old in ((sets, old_sets), (tables, old_tables), (proof_sets, old_proof)):
            for curve in (0, 1):
                for lg, c in old[curve].items():
                    new[curve].setdefault(lg, c)
    gpu = torch.cuda.get_device_name(0)
    with open(args.out, "w") as f:
        f.write(header_text(sets, tables, gpu, proof_sets))
    with open(os.path.splitext(args.out)[0] + ".log", "w") as f:
        f.write("\n".join(log_lines) + "\n")
    ctx.close()


if __name__ == "__main__":
    main()
