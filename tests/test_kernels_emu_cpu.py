"""The PRP kernels' own source compiled for the host and run with one host
thread per GPU thread (tests/emu/), under AddressSanitizer and UBSan:

* the grid kernels (ctwin_gb300/csrc/prp_grid.cu): every CTA of a lane at
  once, the grid barriers, carry counts and polled published words on host
  atomics;
* the one-CTA and cluster kernels (prp_kernel_impl.cuh): the CTAs of a
  cluster at once, cluster barriers and distributed shared memory emulated;
* the whole sieve path (sieve.cu: host driver and kernels, ctw_sieve_run) on
  a stand-in CUDA runtime, CTAs one after another;
* the PRP engine's whole test (prp_engine.cu and its kernels, ctw_prp_run:
  exponent, bit loop, Gerbicz-Li check, canonical digits, RES64) on a
  stand-in runtime that runs clusters and cooperative grids on host threads,
  the server (prp_server.cu over prp_pool.cu: its threads, tick graphs
  recorded and replayed, a slot reused by the next request), the
  allocation-free multiply (prp_noalloc.cu), and a stop at a Gerbicz-Li
  checkpoint with the reference's context file and a resume from it
  (cyclo_files.cu).

Squarings with doubling and one multiply, digits bit-exact with the oracle's C
restatement; struck bitmaps and last p equal to the oracle's sieve; integer
work, tolerance 0.  No GPU involved."""
import os
import re
import shutil
import subprocess

import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
EMU = os.path.join(HERE, "emu")
BUILD = os.path.join(EMU, "_build")
CSRC = os.path.join(ROOT, "ctwin_gb300", "csrc")
# (lg, primes, lm) shapes compiled: 2^16 on 64 CTAs of 1024 (the single-test
# default), 2^16 on 32 CTAs of 2048 with three primes, 2^17 on 32 CTAs of 4096,
# 2^18 on 128 CTAs of 2048 with three primes (the 2^18 default), 2^17 on 64 CTAs
# of 2048 (the 2^17 default)
SHAPES = [(6, 2, 10), (5, 3, 11), (5, 2, 12), (7, 3, 11), (6, 2, 11), (7, 2, 11)]
MARK = "size_t prp_grid_smem_bytes(int lg, int lm, int tw_smem, int np)"


# AddressSanitizer and UBSan on by default; CTW_EMU_FAST=1 builds without them
SAN = [] if os.environ.get("CTW_EMU_FAST") else ["-fsanitize=address,undefined", "-fno-omit-frame-pointer"]


def _compile(exe, sources, shapes_macro):
    lib = O.build()
    cmd = ["g++", "-std=c++20", "-O1", "-g", *SAN, "-I", os.path.join(EMU, "stub"), "-I", EMU, "-I", CSRC,
           "-include", "emu_shim.h", f"-DCTW_EMU_SHAPES={shapes_macro}", "-o", exe, *sources,
           lib, f"-Wl,-rpath,{os.path.dirname(lib)}", "-lpthread"]
    subprocess.run(cmd, check=True, timeout=900)
    return exe


def _run(args):
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([str(v) for v in args], capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "status 0 mismatches square 0 mul 0" in r.stdout


@pytest.fixture(scope="module")
def grid_emu():
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    os.makedirs(BUILD, exist_ok=True)
    src = open(os.path.join(CSRC, "prp_grid.cu")).read()
    cut = src.find(MARK)
    assert cut > 0, "prp_grid.cu: host launch code not found"
    body = src[:cut]
    decl = "extern __shared__ __align__(16) uint32_t sm[];"
    assert body.count(decl) == 2                       # prp_kernel_grid and prp_kernel_grid2
    body = body.replace(decl, "uint32_t *sm = emu_smem();")
    # 1024- and 2048-coefficient CTAs run the warp-local kernel, 4096 the radix-16 one
    kname = lambda lm: "prp_kernel_grid2" if lm <= 11 else "prp_kernel_grid"
    inst = "".join(f"template void {kname(lm)}<{lg}, {np}, {lm}>(const PrpKernelArgs, const PrpGridArgs);\n"
                   for lg, np, lm in SHAPES)
    kern = os.path.join(BUILD, "grid_kernels.cpp")
    with open(kern, "w") as f:
        f.write('#include "emu_shim.h"\n' + body + inst + "}  // namespace ctw\n")
    shapes = " ".join(f"CTW_EMU_SHAPE({lg}, {np}, {lm}, {kname(lm)})" for lg, np, lm in SHAPES)
    return _compile(os.path.join(BUILD, "grid_emu"), [kern, os.path.join(EMU, "grid_emu.cpp")], shapes)


@pytest.mark.parametrize("ln,lm,primes,csize,b,threads,mult", [
    (16, 10, 2, 16, 1330358, 64, 3),     # the 2^16 single-test shape, two primes, Fermat base 3
    (16, 10, 2, 8, 1330358, 64, 3),      # the same with CSIZE 8 (the unrolled carry chain)
    (16, 11, 3, 32, 2000000003, 64, 2),  # three primes, b near 2^31 (128-bit carries)
    (17, 12, 2, 8, 1330358, 32, 2),      # 4096-coefficient CTAs
    (17, 11, 2, 16, 1330358, 64, 2),     # the 2^17 default: 64 CTAs of 2048, runs of 32 columns
    (18, 11, 3, 16, 1330358, 32, 3),     # 128 CTAs
    (18, 11, 2, 8, 1330358, 32, 2),      # 128 CTAs on two primes: the neighbour's chunk through three cross passes
])
def test_grid_kernel_emulated_bit_exact(grid_emu, ln, lm, primes, csize, b, threads, mult):
    _run([grid_emu, ln, lm, primes, csize, b, threads, mult])


# (cols, lg, m12, primes, dense) instantiations of prp_kernel / prp_kernel_cols
CLUSTER_SHAPES = [(0, 0, 0, 2, 0), (0, 0, 1, 3, 0), (1, 2, 1, 2, 0), (1, 1, 1, 3, 1), (1, 2, 0, 3, 0), (0, 0, 1, 2, 0)]
IMPL_MARK = "template <int LG, bool M12, bool COLS, int NP, bool DENSE = false>\nstatic cudaError_t launch_lg"


@pytest.fixture(scope="module")
def cluster_emu():
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    os.makedirs(BUILD, exist_ok=True)
    src = open(os.path.join(CSRC, "prp_kernel_impl.cuh")).read()
    cut = src.find(IMPL_MARK)
    assert cut > 0, "prp_kernel_impl.cuh: launch_lg not found"
    body = src[:cut]
    decl = "extern __shared__ __align__(16) uint32_t sm[];"
    assert body.count(decl) == 2
    body = body.replace(decl, "uint32_t *sm = emu_smem();")
    cu = open(os.path.join(CSRC, "prp_kernels.cu")).read()
    i0, i1 = cu.find("size_t prp_smem_bytes("), cu.find("// Cluster splits with a kernel")
    assert 0 < i0 < i1, "prp_kernels.cu: shared-memory / thread helpers not found"
    tf = lambda v: "true" if v else "false"
    inst = "".join(f"template void {'prp_kernel_cols' if c else 'prp_kernel'}<{lg}, {tf(m)}, {np}, {tf(d)}>"
                   f"(const PrpKernelArgs);\n" for c, lg, m, np, d in CLUSTER_SHAPES)
    kern = os.path.join(BUILD, "cluster_kernels.cpp")
    with open(kern, "w") as f:
        f.write('#include "emu_shim.h"\n' + body + "\n" + cu[i0:i1] + inst + "}  // namespace ctw\n")
    shapes = " ".join(f"CTW_EMU_SHAPE({c}, {lg}, {tf(m)}, {np}, {tf(d)})" for c, lg, m, np, d in CLUSTER_SHAPES)
    return _compile(os.path.join(BUILD, "cluster_emu"), [kern, os.path.join(EMU, "cluster_emu.cpp")], shapes)


@pytest.mark.parametrize("ln,lg,primes,dense,csize,b0,b1", [
    (11, 0, 2, 0, 16, 100003, 299993),       # one CTA of 2048, two primes (the twin-search degree)
    (12, 0, 3, 0, 8, 2000000003, 65537),     # one CTA of 4096, three primes, b near 2^31
    (14, 2, 2, 0, 32, 1330358, 70001),       # 4-CTA cluster of 4096, two primes
    (13, 1, 3, 1, 16, 1330358, 4000037),     # 2-CTA cluster, dense three-prime build (384 threads)
    (13, 2, 3, 0, 8, 2000000011, 100003),    # 4-CTA cluster of 2048, generic three-prime path
])
def test_cluster_kernels_emulated_bit_exact(cluster_emu, ln, lg, primes, dense, csize, b0, b1):
    _run([cluster_emu, ln, lg, primes, dense, csize, b0, b1])


@pytest.mark.parametrize("primes,mult", [(2, 2), (2, 3), (3, 3)])
def test_minus_kernel_emulated(cluster_emu, primes, mult):
    """N- of degree 2^11 on the 4096-coefficient transform (the fold of the
    upper half in the kernel): after one squaring with the base multiplier the
    register is mult x0^2 mod N-, after the multiply x1 y mod N-; the upper
    halves stay zero."""
    b0, b1 = 100019, 299993
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([str(v) for v in (cluster_emu, 12, 0, primes, 0, 16, b0, b1, 1, mult)],
                       capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().split("\n")
    assert lines[-1] == "status 0"
    Dn = 1 << 11
    for lane, b in enumerate((b0, b1)):
        x0, y, x1, out = ([int(v) for v in lines[4 * lane + k].split()] for k in range(4))
        N = b ** Dn - b ** (Dn // 2) - 1
        assert not any(x1[Dn:]) and not any(out[Dn:])
        want1 = mult * O.digits_to_int(x0, b) ** 2 % N
        assert O.digits_to_int(x1, b) % N == want1
        assert O.digits_to_int(out, b) % N == want1 * O.digits_to_int(y, b) % N


SIEVE_LAUNCH = re.compile(r"([A-Za-z_]\w*(?:<[^<>;()]*>)?)<<<(.*?)>>>\(")


@pytest.fixture(scope="module")
def sieve_emu():
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    os.makedirs(BUILD, exist_ok=True)
    src = open(os.path.join(CSRC, "sieve.cu")).read()
    decl = "extern __shared__ uint32_t sbits[];"
    assert src.count(decl) == 2
    src = src.replace(decl, "uint32_t *sbits = emu_dyn_smem();")
    src, k = SIEVE_LAUNCH.subn(lambda m: f"emu_launch({m.group(1)}, EmuCfg{{{m.group(2)}}})(", src)
    assert k > 0 and "<<<" not in src
    gen = os.path.join(BUILD, "sieve_src.cpp")
    with open(gen, "w") as f:
        f.write(src)
    exe = os.path.join(BUILD, "sieve_emu")
    cmd = ["g++", "-std=c++20", "-O1", "-g", *SAN, "-I", os.path.join(EMU, "sieve_stub"), "-I", EMU, "-I", CSRC,
           "-o", exe, gen, os.path.join(EMU, "sieve_emu.cpp"), "-lpthread"]
    subprocess.run(cmd, check=True, timeout=900)
    return exe


@pytest.mark.parametrize("n,b_min,b_max,p_min,p_max,mode", [
    (8, 2, 2000, 769, 10 ** 6, 1),
    (8, 2, 2, 11, 10 ** 5, -1),                                  # a single b
    (12, 5, 20000, 11, 10 ** 6, -1),                             # 32-bit Montgomery path
    (11, 2, 10 ** 6, 2 ** 32 - 10 ** 7, 2 ** 32 + 10 ** 7, 1),   # p across 2^32
    (12, 5, 20000, 2 ** 32 - 10 ** 6, 2 ** 32 + 10 ** 6, -1),    # 64-bit path of the - form
])
def test_sieve_emulated_matches_oracle(sieve_emu, n, b_min, b_max, p_min, p_max, mode):
    import numpy as np
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([str(v) for v in (sieve_emu, n, b_min, b_max, p_min, p_max, mode)],
                       capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stdout[:500] + r.stderr[-2000:]
    head, words = r.stdout.strip().split("\n")[:2]
    p_last = int(head.split()[3])
    w = np.array([int(v) for v in words.split()], dtype=np.uint32)
    got = np.unpackbits(w.view(np.uint8), bitorder="little")[: b_max - b_min + 1]
    want, want_last = O.sieve(n, b_min, b_max, p_min, p_max, mode, threads=8)
    assert np.array_equal(got, want)
    assert p_last == want_last


@pytest.mark.parametrize("name", ["n8_small", "n9_small"])
def test_sieve_emulated_matches_reference_files(sieve_emu, golden_dir, name, tmp_path):
    """A reference sieve case run through the emulated product path: the last p
    of each form and the md5 of the sv_*.dat / cand_*.txt files equal the
    reference CPU sieve's own (tests/golden/sieve_files.json)."""
    import hashlib
    import json
    meta = json.load(open(os.path.join(golden_dir, "sieve_files.json")))
    m = meta["cases"][name]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([str(v) for v in (sieve_emu, "case", m["n"], m["b_min"], m["b_max"], m["p_max_pos"],
                                         m["p_max_neg"], m["mode"], tmp_path)],
                       capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stdout[:500] + r.stderr[-2000:]
    _, _, _, p_pos, p_neg = r.stdout.split()[:5]
    if m["mode"] >= 0:
        assert int(p_pos) == m["p_last_pos"]
    if m["mode"] <= 0:
        assert int(p_neg) == m["p_last_neg"]
    files = meta["files"][name]
    assert files
    for fname, md5 in files.items():
        assert hashlib.md5((tmp_path / fname).read_bytes()).hexdigest() == md5, fname


@pytest.mark.parametrize("mode", [1, -1])
def test_sieve_factors_emulated(sieve_emu, mode):
    """ctw_sieve_factors (the GPU sieve's factor pairs) on the emulated path:
    every pair divides, pairs are sorted by p, and the set of b is the set the
    oracle's sieve strikes over the same primes."""
    import numpy as np
    from ctwin_gb300.gfsieve import divides
    n, b_max = 8, 1 << 16
    if mode > 0:
        k_b, k_e = 1 << 14, (1 << 14) + (1 << 10)
        p_min, p_max = 3 * (k_b << n) + 1, 3 * ((k_e - 1) << n) + 1
    else:
        k_b, k_e = 1 << 16, (1 << 16) + (1 << 10)
        p_min, p_max = 10 * k_b, 10 * (k_e - 1)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([str(v) for v in (sieve_emu, "factors", n, k_b, k_e, mode, b_max)],
                       capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stdout[:500] + r.stderr[-2000:]
    lines = r.stdout.strip().split("\n")
    count = int(lines[0].split()[3])
    pairs = [tuple(map(int, l.split())) for l in lines[1:1 + count]]
    assert count > 0 and len(pairs) == count
    assert all(p > b_max for p, _ in pairs)
    assert all(divides(p, b, n, mode) for p, b in pairs)
    assert all(pairs[i][0] <= pairs[i + 1][0] for i in range(count - 1))
    bits, _ = O.sieve(n, 2, b_max, p_min, p_max, mode, threads=8)
    assert {b for _, b in pairs} == {int(b) for b in np.flatnonzero(bits) + 2}


ENGINE_SOURCES = ("prp_engine.cu", "prp_kernels.cu", "prp_kernels_np2.cu", "prp_grid.cu", "prp_pool.cu",
                  "prp_batch.cu", "prp_server.cu", "prp_noalloc.cu", "cyclo_files.cu")


@pytest.fixture(scope="module")
def engine_emu():
    """The engine's sources with their launches rewritten as calls, compiled
    without sanitizers (a whole test is thousands of launches)."""
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    b = os.path.join(BUILD, "engine")
    os.makedirs(b, exist_ok=True)
    decl = "extern __shared__ __align__(16) uint32_t sm[];"
    for f in ENGINE_SOURCES + ("prp_kernel_impl.cuh",):
        src = open(os.path.join(CSRC, f)).read().replace(decl, "uint32_t *sm = emu_smem();")
        src = SIEVE_LAUNCH.sub(lambda m: f"emu_launch({m.group(1)}, EmuCfg{{{m.group(2)}}})(", src)
        assert "<<<" not in src
        with open(os.path.join(b, f[:-3] + ".cpp" if f.endswith(".cu") else f), "w") as fh:
            fh.write(src)
    flags = ["-std=c++20", "-O1", "-I", os.path.join(EMU, "engine_stub"), "-I", os.path.join(EMU, "stub"), "-I", EMU,
             "-I", CSRC, "-include", "emu_shim.h"]
    objs = []
    procs = []
    for f in ENGINE_SOURCES:
        o = os.path.join(b, f[:-3] + ".o")
        objs.append(o)
        procs.append(subprocess.Popen(["g++", *flags, "-c", "-o", o, os.path.join(b, f[:-3] + ".cpp")]))
    assert all(p.wait(timeout=900) == 0 for p in procs)
    exe = os.path.join(b, "engine_emu")
    subprocess.run(["g++", *flags, "-o", exe, os.path.join(EMU, "engine_emu.cpp"), *objs, "-lpthread"], check=True,
                   timeout=900)
    return exe


@pytest.mark.parametrize("b,base,form", [(68, 3, "+"), (68, 2, "-")])
def test_engine_whole_test_emulated_matches_gmp(engine_emu, golden_dir, b, base, form):
    """ctw_prp_run of one candidate of degree 2^8 (N- on the 2^9 transform) on
    the emulated engine: PRP flag and RES64 equal GMP's, Gerbicz-Li check passes."""
    import json
    want = next(x for x in json.load(open(os.path.join(golden_dir, "prp_gmp.json")))
                if x["n"] == 8 and x["b"] == b and x["base"] == base and x["form"] == form)
    r = subprocess.run([engine_emu, "8", str(base), "1" if form == "-" else "0", str(b)],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    got_b, prp, res64, gl = r.stdout.split()[:4]
    assert int(got_b) == b and gl == "1"
    assert (prp == "1", res64) == (want["prp"], want["res64"])


def test_server_emulated_matches_gmp(engine_emu, golden_dir):
    """The request loop (prp_server.cu: preparation and worker threads over
    pools) with one slot: two base-3 requests of degree 2^8, the second
    admitted when the first retires, tick graphs recorded and replayed.
    PRP flags, RES64 and Gerbicz-Li checks equal GMP's, one of them a PRP."""
    import json
    gold = {x["b"]: x for x in json.load(open(os.path.join(golden_dir, "prp_gmp.json")))
            if x["n"] == 8 and x["base"] == 3 and x["form"] == "+"}
    bs = [68, 298]
    r = subprocess.run([engine_emu, "server", "8", "1", "3", *map(str, bs)], capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    got = {}
    for line in r.stdout.strip().splitlines():
        b, prp, res64, gl, status, slot = line.split()
        got[int(b)] = (prp == "1", res64, gl, status)
    assert sorted(got) == bs
    for b in bs:
        assert got[b] == (gold[b]["prp"], gold[b]["res64"], "1", "0"), b
    assert any(gold[b]["prp"] for b in bs)


@pytest.mark.parametrize("lanes", [1, 2])
def test_server_grid_lane_emulated_matches_gmp(engine_emu, golden_dir, lanes):
    """The server's grid lane (a thread running one test at a time on a
    one-lane engine, taking turns on the device with the pools at every
    Gerbicz-Li checkpoint), threshold 2^9 for the emulation (2^16 by default):
    two requests of degree 2^9 in one lane (first come, first served) or in
    two (their one-CTA grids fit the device together) while two of 2^8 share
    a one-slot pool.  PRP flags and RES64 equal GMP's on both paths; the
    lanes' results carry slot -2."""
    import json
    gold = {x["b"]: x for x in json.load(open(os.path.join(golden_dir, "prp_gmp.json")))
            if x["n"] == 8 and x["base"] == 3 and x["form"] == "+"}
    bs = [68, 298]
    lane_bs = [71, 79]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0", CTW_EMU_GRID_LANE="9:" + ",".join(map(str, lane_bs)),
               CTW_EMU_GRID_LANES=str(lanes))
    r = subprocess.run([engine_emu, "server", "8", "1", "3", *map(str, bs)], capture_output=True, text=True,
                       timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    got = {}
    for line in r.stdout.strip().splitlines():
        b, p, res64, gl, status, slot = line.split()
        got[int(b)] = (p == "1", res64, gl, status, int(slot))
    assert sorted(got) == sorted(bs + lane_bs)
    for b in bs:
        assert got[b][:4] == (gold[b]["prp"], gold[b]["res64"], "1", "0"), b
        assert got[b][4] >= 0
    for b in lane_bs:
        _, r64, prp = O.fermat(b, 9, 3)
        assert got[b] == (prp, f"{r64:016X}", "1", "0", -2), b


def test_batch_emulated_equals_pools(engine_emu):
    """A batch of pools of degrees 2^12 (two and three primes), 2^13 and 2^14
    (prp_pool.cu's batch ticks: every pool's squarings in one persistent launch
    of clusters of 8 CTAs with per-degree queues, prp_batch.cu) against the
    same pools ticked on their own: every register of every slot equal after
    two ticks of 8 squarings and a multiply (base 3)."""
    r = subprocess.run([engine_emu, "batch", "2"], capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout + r.stderr[-2000:]
    assert " differ 0" in r.stdout


@pytest.mark.parametrize("ln,bs,csize", [(11, [100003, 299993], 16), (13, [1330358], 8)])
def test_mul_noalloc_emulated_bit_exact(engine_emu, tmp_path, ln, bs, csize):
    """ctw_prp_mul_noalloc (fixed device arrays, no allocation) on the emulated
    runtime: z = x * y digits bit-exact with the oracle's multiply."""
    import numpy as np
    rng = np.random.default_rng(ln)
    D = 1 << ln
    x = np.stack([rng.integers(-(b // 2), b // 2, D, dtype=np.int64) for b in bs]).astype(np.int32)
    y = np.stack([rng.integers(-(b // 2), b // 2, D, dtype=np.int64) for b in bs]).astype(np.int32)
    fin, fout = tmp_path / "xy.bin", tmp_path / "z.bin"
    np.concatenate([x.ravel(), y.ravel()]).tofile(fin)
    r = subprocess.run([engine_emu, "mul", str(ln), str(csize), str(fin), str(fout), *map(str, bs)],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    z = np.fromfile(fout, dtype=np.int32).reshape(len(bs), D)
    with O.Tables(ln) as t:
        for lane, b in enumerate(bs):
            w = x[lane].copy()
            t.mul(w, y[lane].copy(), b, csize)
            assert np.array_equal(z[lane], w), lane


def test_context_stop_and_resume_emulated(engine_emu, golden_dir, tmp_path):
    """A whole base-3 test of degree 2^8 stops at its first Gerbicz-Li
    checkpoint and saves the reference's context file there
    (ctw_prp_save_context); a fresh engine reads it (ctw_prp_read_context)
    and resumes (ctw_prp_run_ex from the saved bit): the verdict and RES64
    equal GMP's (a PRP)."""
    import json
    want = next(x for x in json.load(open(os.path.join(golden_dir, "prp_gmp.json")))
                if x["n"] == 8 and x["b"] == 298 and x["base"] == 3 and x["form"] == "+")
    ctx = tmp_path / "cyclo.ctx"
    r = subprocess.run([engine_emu, "resume", "8", "3", str(ctx), "298"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    b, prp, res64, gl, i_stop = r.stdout.split()
    assert int(b) == 298 and gl == "1" and int(i_stop) > 0
    assert (prp == "1", res64) == (want["prp"], want["res64"])
    assert ctx.exists()
