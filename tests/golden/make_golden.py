"""Generate the golden fixtures under tests/golden/ (run once, in a container that
has the reference source; the outputs are committed, the GPU tests only read them).

  algo_kat.json     known-answer squares mod X^n - X^{n/2} + 1 for n = 8, 16, parsed
                    from the reference's own check strings (cyclo/algo/algo.cpp:173-177)
  sieve_ref.npz     survivor bitmaps + last p of the reference CPU sieve itself
                    (sieve/CPU/ctsieve.cpp, compiled unchanged into oracle/_ref/)
  sieve_files.json  md5 of cand_*.txt / sv_*.dat written by the reference's write(true)
  prp_gmp.json      GMP Fermat residues (RES64, PRP flag) for base 2 and 3, N+ and N-
  pool_gmp.json     GMP Fermat residues of the pool / server cases (degrees 2^9..2^15)
  prp16_gmp.json    degree 2^16: whole Fermat tests of small b (N+ base 2 and 3, N-),
                    and r_K = base^(E >> (L - K)) mod N+ for K = 4096 at the single-test
                    workload's b (sha256 of the residue's little-endian bytes + its low 64 bits)
  prefix_gmp.json   the same 4096-squaring prefix at degrees 2^17 and 2^18 (the grid
                    kernel on two and three primes), base 2
  prefix64k_gmp.json  r_K for K = 65536 at degree 2^16 and the single-test workload's b,
                    base 3 (the Fermat base of that workload)
  sieve_cfg4.json   the large sieve (n = 20, p = 3k 2^20 + 1 up to 2^40, + form) of the
                    reference CPU sieve over four seeded sub-ranges [s, s + 2^24) of
                    [2, 2^30): sha256 of the packed survivor bitmap, survivor count, last p
                    and md5 of sv_*.dat / cand_*.txt; the p range is cut into k slices run
                    in parallel (the reference's own resume by _p_min_pos) and OR-ed

Usage:  CTWIN_REFERENCE=<reference checkout> python tests/golden/make_golden.py
            [--skip-slow] [--only pool|big|prefix|cfg1|cfg4]
  (--only cfg1 extends prp_gmp.json to the first 256 twin survivors at n = 11:
   N+ base 2 and 3, N- base 2 and 3)
"""
from __future__ import annotations

import argparse
import hashlib
import json
import multiprocessing as mp
import os
import re
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = os.environ.get("CTWIN_REFERENCE", "")


def ref_dir() -> str:
    if not REF or not os.path.isdir(REF):
        sys.exit("set CTWIN_REFERENCE to the reference checkout (the directory holding cyclo/ and sieve/)")
    return REF


def algo_kat():
    src = open(os.path.join(ref_dir(), "cyclo", "algo", "algo.cpp")).read()
    out = {}
    for n, rhs in re.findall(r'check\((\d+),\s*"\s*=\s*([^"]+)"\)', src):
        n = int(n)
        coeffs = [0] * n
        for sign, mag, power in re.findall(r'([+-]?)\s*(\d+)(\*x(?:\^\d+)?)?', rhs.replace(" ", "")):
            e = 0 if not power else (1 if power == "*x" else int(power.split("^")[1]))
            coeffs[e] = -int(mag) if sign == "-" else int(mag)
        out[str(n)] = coeffs
    return out


SIEVE_CASES = [
    # name, n, b_min, b_max(inclusive), p_max_pos, p_max_neg, mode
    ("cfg1_pos", 11, 100000, 299999, 2 ** 32, 11, 1),
    ("cfg1_twin", 11, 100000, 299999, 2 ** 32, 2 ** 32, 0),
    ("n8_small", 8, 2, 20000, 10 ** 7, 10 ** 6, 0),
    ("n9_small", 9, 2, 3, 10 ** 6, 10 ** 6, 0),
    ("n10_mid", 10, 50000, 70000, 2 ** 34, 2 ** 28, 0),
    ("n12_pos", 12, 2, 200000, 2 ** 36, 11, 1),
    ("n14_pos", 14, 123456, 223455, 2 ** 36, 11, 1),
    ("n16_pos", 16, 2, 65537, 2 ** 36, 11, 1),
    ("n20_pos_s0", 20, 2, 2 ** 16, 2 ** 36, 11, 1),
]


def run_sieve_case(case):
    from oracle import oracle as O
    name, n, bmin, bmax, pp, pn, mode = case
    tmp = tempfile.mkdtemp()
    r = O.ref_sieve(n, bmin, bmax, pp, pn, mode, write_dir=tmp)
    files = {}
    for f in os.listdir(tmp):
        files[f] = hashlib.md5(open(os.path.join(tmp, f), "rb").read()).hexdigest()
    return name, r, files


def prp_case(args):
    from oracle import oracle as O
    b, ln, base, minus = args
    r, r64, prp = O.fermat(b, ln, base, minus)
    return {"b": b, "n": ln, "base": base, "form": "-" if minus else "+", "res64": f"{r64:016X}", "prp": bool(prp)}


# degree 2^16 whole tests: GMP needs 10-40 minutes each for b < 2^7
BIG_FULL = [(65, 16, 2, False), (100, 16, 2, False), (127, 16, 2, False), (100, 16, 3, False), (101, 16, 2, True)]
# b of the single-test workload (b uniform in [2^20, 2^21), seed 1) and the prefix length
BIG_PARTIAL_B, BIG_PARTIAL_K = 1330358, 4096


def partial_case(args):
    from oracle import oracle as O
    b, ln, base, K = args
    N = O.n_plus(b, ln)
    E = N - 1
    r = O.powmod(base, E >> (E.bit_length() - K), N)
    raw = r.to_bytes((N.bit_length() + 7) // 8, "little")
    return {"b": b, "n": ln, "base": base, "form": "+", "K": K, "sha256": hashlib.sha256(raw).hexdigest(),
            "low64": f"{r & (2 ** 64 - 1):016X}"}


def big_case(job):
    return partial_case(job[1]) if job[0] == "partial" else prp_case(job[1])


def pool_jobs():
    import random
    jobs = []
    # split / csize coverage at degrees 2^12..2^15 (small b keeps GMP and the GPU quick)
    for ln in (12, 13, 14, 15):
        for b in (64, 65, 100, 1000):
            jobs.append((b, ln, 2, False))
    jobs.append((77, 12, 3, False))
    for ln in (12, 13):
        for b in (65537, 70001, 100003):
            jobs.append((b, ln, 2, False))
    jobs.append((65539, 12, 3, False))
    # b on both sides of the two-prime bound 3 D (b + 1)^2 < q0 q1 at degrees 2^12 and 2^13
    for ln, bs in ((12, (9000001, 9999991, 16777213)), (13, (6500003, 6700001))):
        for b in bs:
            jobs.append((b, ln, 2, False))
    # server mixes: seeded b in [2^16, 2^20) at degrees 2^9..2^11
    rng = random.Random(5)
    for ln in (9, 10, 11):
        for _ in range(24):
            jobs.append((rng.randrange(1 << 16, 1 << 20), ln, 2, False))
    return jobs


# the large sieve: n = 20, b in [2, 2^30), p = 3k 2^20 + 1 < 2^40, + form
CFG4_N, CFG4_SPAN, CFG4_P_MAX, CFG4_SEED, CFG4_RANGES, CFG4_SLICES = 20, 1 << 24, 1 << 40, 20, 4, 16


def cfg4_starts() -> list[int]:
    import random
    rng = random.Random(CFG4_SEED)
    return [rng.randrange(2, (1 << 30) - CFG4_SPAN + 1) for _ in range(CFG4_RANGES)]


def cfg4_slices() -> list[tuple[int, int]]:
    """(p_min, p_max) per k slice.  check_pos runs k from (p_min >> n) / 3 to the
    first k with 3 k 2^n + 1 >= p_max (ctsieve.cpp:680-681), so slices of whole k
    with p_min = 3 k0 2^n + 1 and p_max = 3 (k1 - 1) 2^n + 1 are disjoint; the last
    one keeps p_max = 2^40 and with it the reference's k past the limit."""
    n = CFG4_N
    k_lo = 1
    k_hi = (CFG4_P_MAX >> n) // 3
    while 3 * (k_hi << n) + 1 < CFG4_P_MAX:
        k_hi += 1
    # equal numbers of primes per slice, roughly: cut the k range evenly
    cuts = [k_lo + (k_hi + 1 - k_lo) * i // CFG4_SLICES for i in range(CFG4_SLICES + 1)]
    out = []
    for i in range(CFG4_SLICES):
        k0, k1 = cuts[i], cuts[i + 1]
        p_max = CFG4_P_MAX if i == CFG4_SLICES - 1 else 3 * ((k1 - 1) << n) + 1
        out.append((3 * (k0 << n) + 1, p_max))
    return out


def cfg4_job(job):
    from oracle import oracle as O
    s, p_min, p_max = job
    tmp = tempfile.mkdtemp()
    cwd = os.getcwd()
    os.chdir(tmp)               # the reference's periodic write(false) lands here
    try:
        bits, lp, _ = O.ref_sieve(CFG4_N, s, s + CFG4_SPAN - 1, p_max, 11, 1, p_min_pos=p_min)
    finally:
        os.chdir(cwd)
    return s, p_min, np.packbits(bits, bitorder="little"), lp


def cfg4():
    from oracle import oracle as O
    O.build_ref(ref_dir())
    jobs = [(s, a, b) for s in cfg4_starts() for a, b in cfg4_slices()]
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        res = pool.map(cfg4_job, jobs)
    out = []
    for s in cfg4_starts():
        mine = sorted((r for r in res if r[0] == s), key=lambda r: r[1])
        packed = np.bitwise_or.reduce(np.stack([r[2] for r in mine]), axis=0)
        p_last = mine[-1][3]
        bits = np.unpackbits(packed, bitorder="little")[:CFG4_SPAN]
        surv = np.flatnonzero(bits == 0)
        b_max = s + CFG4_SPAN - 1
        sv = O.sv_bytes(bits, p_last, 11)
        cand = O.cand_text(bits, s).encode()
        out.append({"n": CFG4_N, "b_min": s, "b_max": b_max, "p_min_pos": 3 * (1 << CFG4_N) + 1,
                    "p_max_pos": CFG4_P_MAX, "p_last_pos": p_last, "survivors": int(surv.size),
                    "sha256_bits": hashlib.sha256(packed.tobytes()).hexdigest(),
                    "first_survivors": [s + int(i) for i in surv[:64]],
                    "files": {f"sv_{CFG4_N}_{s}_{b_max}.dat": hashlib.md5(sv).hexdigest(),
                              f"cand_{CFG4_N}_{s}_{b_max}.txt": hashlib.md5(cand).hexdigest()}})
        print(s, p_last, surv.size, flush=True)
    json.dump({"seed": CFG4_SEED, "span": CFG4_SPAN, "slices": CFG4_SLICES, "ranges": out},
              open(os.path.join(HERE, "sieve_cfg4.json"), "w"), indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--skip-slow", action="store_true")
    ap.add_argument("--only", choices=["pool", "big", "prefix", "prefix64k", "cfg1", "cfg4"], default=None)
    args = ap.parse_args()
    from oracle import oracle as O
    O.build()
    if args.only == "cfg4":
        cfg4()
        return
    if args.only == "prefix64k":
        res = [partial_case((BIG_PARTIAL_B, 16, 3, 65536))]
        json.dump(res, open(os.path.join(HERE, "prefix64k_gmp.json"), "w"), indent=0)
        print("done", res)
        return
    if args.only == "cfg1":
        path = os.path.join(HERE, "prp_gmp.json")
        old = json.load(open(path))
        have = {(d["b"], d["n"], d["base"], d["form"] == "-") for d in old}
        z = np.load(os.path.join(HERE, "sieve_ref.npz"))
        meta = json.load(open(os.path.join(HERE, "sieve_files.json")))["cases"]["cfg1_twin"]
        twin = np.unpackbits(z["cfg1_twin"], bitorder="little")[: meta["size"]]
        surv = [meta["b_min"] + int(i) for i in np.flatnonzero(twin == 0)[:256]]
        jobs = [(b, 11, base, minus) for b in surv for base in (2, 3) for minus in (False, True)]
        todo = [j for j in jobs if j not in have]
        with mp.get_context("spawn").Pool(min(8, os.cpu_count() or 1)) as pool:
            new = pool.map(prp_case, todo)
        json.dump(old + new, open(path, "w"), indent=0)
        print("added", len(new), "config-1 cases")
        return
    if args.only == "prefix":
        jobs = [(BIG_PARTIAL_B, ln, 2, BIG_PARTIAL_K) for ln in (17, 18)]
        with mp.get_context("spawn").Pool(len(jobs)) as pool:
            res = pool.map(partial_case, jobs)
        json.dump(res, open(os.path.join(HERE, "prefix_gmp.json"), "w"), indent=0)
        print("done", len(res), "prefix cases")
        return
    if args.only == "big":
        jobs = [("partial", (BIG_PARTIAL_B, 16, base, BIG_PARTIAL_K)) for base in (2, 3)]
        jobs += [("full", j) for j in BIG_FULL]
        with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
            res = pool.map(big_case, jobs)
        json.dump(res, open(os.path.join(HERE, "prp16_gmp.json"), "w"), indent=0)
        print("done", len(res), "degree-2^16 cases")
        return
    if args.only == "pool":
        path = os.path.join(HERE, "pool_gmp.json")
        have = {}
        if os.path.exists(path):
            have = {(d["b"], d["n"], d["base"], d["form"] == "-"): d for d in json.load(open(path))}
        todo = [j for j in pool_jobs() if j not in have]
        with mp.get_context("spawn").Pool(min(8, os.cpu_count() or 1)) as pool:
            new = pool.map(prp_case, todo)
        res = [have[j] if j in have else new[todo.index(j)] for j in pool_jobs()]
        json.dump(res, open(os.path.join(HERE, "pool_gmp.json"), "w"), indent=0)
        print("done", len(res), "pool cases")
        return
    O.build_ref(ref_dir())

    json.dump(algo_kat(), open(os.path.join(HERE, "algo_kat.json"), "w"), indent=1)

    cases = SIEVE_CASES if not args.skip_slow else [c for c in SIEVE_CASES if c[0] != "cfg1_twin"]
    with mp.get_context("spawn").Pool(min(8, os.cpu_count() or 1)) as pool:
        res = pool.map(run_sieve_case, cases)
    arrays, meta, files = {}, {}, {}
    for (name, r, fl), case in zip(res, cases):
        bits, lp, ln_ = r
        arrays[name] = np.packbits(bits, bitorder="little")
        meta[name] = {"n": case[1], "b_min": case[2], "b_max": case[3], "p_max_pos": case[4], "p_max_neg": case[5],
                      "mode": case[6], "p_last_pos": lp, "p_last_neg": ln_, "size": int(bits.size),
                      "survivors": int((bits == 0).sum())}
        files[name] = fl
    np.savez_compressed(os.path.join(HERE, "sieve_ref.npz"), **arrays)
    json.dump({"cases": meta, "files": files}, open(os.path.join(HERE, "sieve_files.json"), "w"), indent=1)

    # PRP residues: survivors of config 1 (twin list), small-n PRP hunts, base 2 and 3, N+ and N-
    twin = np.unpackbits(arrays["cfg1_twin"], bitorder="little")[: meta["cfg1_twin"]["size"]] if "cfg1_twin" in arrays else None
    jobs = []
    if twin is not None:
        surv = [100000 + int(i) for i in np.flatnonzero(twin == 0)[:64]]
        for b in surv:
            for base in (2, 3):
                jobs.append((b, 11, base, False))
            jobs.append((b, 11, 2, True))
    small = np.unpackbits(arrays["n8_small"], bitorder="little")[: meta["n8_small"]["size"]]
    s8 = [2 + int(i) for i in np.flatnonzero(small == 0)]
    for b in s8[:400]:
        if b >= 64:
            jobs.append((b, 8, 2, False))
            jobs.append((b, 8, 3, False))
            jobs.append((b, 8, 2, True))
    with mp.get_context("spawn").Pool(min(8, os.cpu_count() or 1)) as pool:
        prp = pool.map(prp_case, jobs)
    json.dump(prp, open(os.path.join(HERE, "prp_gmp.json"), "w"), indent=0)
    print("done", len(prp), "prp cases;", sum(p["prp"] for p in prp), "PRPs")


if __name__ == "__main__":
    main()
