"""The grid kernel's own source (ctwin_gb300/csrc/prp_grid.cu) compiled for the
host and run with one host thread per GPU thread (tests/emu/): every CTA of a
lane at once, the grid barriers and the neighbour carry publications on host
atomics, under AddressSanitizer and UBSan.  Two doubling squarings and one
multiply, digits bit-exact with the oracle's C restatement; integer work,
tolerance 0.  No GPU involved."""
import os
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
# default), 2^16 on 32 CTAs of 2048 with three primes, 2^17 on 32 CTAs of 4096
SHAPES = [(6, 2, 10), (5, 3, 11), (5, 2, 12)]
MARK = "size_t prp_grid_smem_bytes(int lg, int lm, int tw_smem, int np)"


@pytest.fixture(scope="module")
def grid_emu():
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    lib = O.build()
    os.makedirs(BUILD, exist_ok=True)
    src = open(os.path.join(CSRC, "prp_grid.cu")).read()
    cut = src.find(MARK)
    assert cut > 0, "prp_grid.cu: host launch code not found"
    body = src[:cut]
    decl = "extern __shared__ __align__(16) uint32_t sm[];"
    assert body.count(decl) == 1
    body = body.replace(decl, "uint32_t *sm = emu_smem();")
    inst = "".join(f"template void prp_kernel_grid<{lg}, {np}, {lm}>(const PrpKernelArgs, const PrpGridArgs);\n"
                   for lg, np, lm in SHAPES)
    kern = os.path.join(BUILD, "grid_kernels.cpp")
    with open(kern, "w") as f:
        f.write('#include "emu_shim.h"\n' + body + inst + "}  // namespace ctw\n")
    exe = os.path.join(BUILD, "grid_emu")
    shapes = " ".join(f"CTW_EMU_SHAPE({lg}, {np}, {lm})" for lg, np, lm in SHAPES)
    # AddressSanitizer and UBSan on by default (about 45 s in all); CTW_EMU_FAST=1 builds without them
    san = [] if os.environ.get("CTW_EMU_FAST") else ["-fsanitize=address,undefined", "-fno-omit-frame-pointer"]
    cmd = ["g++", "-std=c++20", "-O1", "-g", *san, "-I", os.path.join(EMU, "stub"), "-I", EMU, "-I", CSRC,
           "-include", "emu_shim.h", f"-DCTW_EMU_SHAPES={shapes}", "-o", exe, kern, os.path.join(EMU, "grid_emu.cpp"),
           lib, f"-Wl,-rpath,{os.path.dirname(lib)}", "-lpthread"]
    subprocess.run(cmd, check=True, timeout=600)
    return exe


@pytest.mark.parametrize("ln,lm,primes,csize,b,threads", [
    (16, 10, 2, 16, 1330358, 64),        # the 2^16 single-test shape, two primes
    (16, 11, 3, 32, 2000000003, 64),     # three primes, b near 2^31 (128-bit carries)
    (17, 12, 2, 8, 1330358, 32),         # 4096-coefficient CTAs
])
def test_grid_kernel_emulated_bit_exact(grid_emu, ln, lm, primes, csize, b, threads):
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([grid_emu, str(ln), str(lm), str(primes), str(csize), str(b), str(threads)],
                       capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "status 0 mismatches square 0 mul 0" in r.stdout
