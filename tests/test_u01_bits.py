"""pcg_u01_bits (integer-only construction of libstdc++'s generate_canonical
double from one 64-bit draw) equals the FP64 conversion it replaces, on edge
cases, rounding ties and random draws. Host code compiled with nvcc; no GPU."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "nqes-trapped-ion_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <cstring>
#include <cmath>
#include <random>
#include "pcg64.cuh"
using namespace nqes;
static uint64_t ref_bits(uint64_t x) {
    double u = double(x) * 0x1p-64;          // round to nearest, exact scaling
    if (u >= 1.0) u = std::nextafter(1.0, 0.0);
    uint64_t b;
    std::memcpy(&b, &u, 8);
    return b;
}
int main() {
    std::vector<uint64_t> xs = {0ULL, 1ULL, 2ULL, 3ULL, (1ULL << 53) - 1, 1ULL << 53, (1ULL << 53) + 1,
                                (1ULL << 63) - 1, 1ULL << 63, (1ULL << 63) + 1, ~0ULL, ~0ULL - 1024, ~0ULL - 2048};
    for (int s = 11; s < 64; s++)
        for (uint64_t lo : {0x3FFULL, 0x400ULL, 0x401ULL, 0xBFFULL, 0xC00ULL, 0xC01ULL}) {
            const uint64_t top = (1ULL << s) | ((0x5A5A5A5A5A5A5A5AULL >> (64 - s)) & ((1ULL << s) - 1));
            xs.push_back(((top >> 11) << 11 | lo) >> (s < 63 ? 0 : 0));
            xs.push_back(((~0ULL >> (63 - s)) & ~0x7FFULL) | lo);
        }
    std::mt19937_64 g(12345);
    for (int t = 0; t < 1000000; t++) xs.push_back(g() >> (t % 64));
    Pcg64 p = pcg_seed(20240601);
    for (int t = 0; t < 200000; t++) xs.push_back(pcg_next(p));
    long bad = 0;
    for (uint64_t x : xs)
        if (pcg_u01_bits(x) != ref_bits(x)) {
            if (bad < 5) std::printf("mismatch x=%016llx got=%016llx want=%016llx\n", (unsigned long long)x,
                                     (unsigned long long)pcg_u01_bits(x), (unsigned long long)ref_bits(x));
            bad++;
        }
    std::printf("checked %zu bad %ld\n", xs.size(), bad);
    return bad != 0;
}
"""


def test_u01_bits_matches_fp64_conversion():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "u01.cu")
        with open(src, "w") as f:
            f.write(PROGRAM)
        exe = os.path.join(d, "u01")
        subprocess.check_call([nvcc, "-std=c++17", "-O2", "-I", CSRC, src, "-o", exe])
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "bad 0" in r.stdout
