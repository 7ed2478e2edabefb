"""The FP32 <-> int64 conversions used by the projection folds, the per-pair
atomics and the FIR staging (openbcsim_gb300/csrc/fixedpoint.cuh) round exactly
like the C library's round-to-nearest-even conversions (llrintf and the int64
-> float cast), over edge values and random bit patterns.  The functions are
plain C++ compiled here for the host (the bounded conversion's device form
swaps nearbyint/floor/fma for the CUDA intrinsics of the same rounding)."""
import os
import subprocess

from conftest import ROOT

PROGRAM = r'''
#include <cfenv>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <random>
#include "fixedpoint.cuh"
using namespace bcsim_gb300;
static float from_bits(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
int main() {
    std::fesetround(FE_TONEAREST);
    long bad = 0, checked = 0;
    std::mt19937_64 rng(12345);
    auto check_f = [&](float x) {
        if (!(std::fabs(x) < 9.2e18f)) return;   // in range of int64
        const long long want = std::llrint((double)x);   // exact: x is representable in double
        const long long got = f2ll_rn(x);
        checked++;
        if (want != got) { if (bad++ < 5) std::printf("f2ll %a want %lld got %lld\n", x, want, got); }
        const long long got_b = f2ll_rn_bounded(x);
        checked++;
        if (want != got_b) { if (bad++ < 5) std::printf("f2ll_bounded %a want %lld got %lld\n", x, want, got_b); }
    };
    auto check_l = [&](long long v) {
        const float want = (float)v;
        const float got = ll2f_rn(v);
        checked++;
        if (std::memcmp(&want, &got, 4) != 0) { if (bad++ < 5) std::printf("ll2f %lld want %a got %a\n", v, want, got); }
    };
    const float edges[] = {0.0f, -0.0f, 0.5f, -0.5f, 1.5f, 2.5f, -2.5f, 0.49999997f, 1e-40f, -1e-40f,
                           8388607.5f, 8388608.0f, 16777215.0f, 16777217.0f, 4.6e18f, -4.6e18f, 9.2e18f,
                           2147483520.0f, 2147483648.0f, -2147483648.0f, -2147483904.0f, 4294967296.0f,
                           -4294967296.0f, 4294967040.0f, -4294967040.0f, 1.5e10f, -1.5e10f, 4.611686e18f,
                           -4.611686e18f, 4.6116855e18f, -4.6116855e18f};
    for (float x : edges) check_f(x);
    for (int i = 0; i < 4000000; i++) {
        unsigned u = (unsigned)rng();
        check_f(from_bits(u));
        // values near half-integers
        const float h = (float)(rng() % 100000000) + 0.5f;
        check_f(h); check_f(-h);
    }
    const long long ledges[] = {0, 1, -1, 16777216, 16777217, 16777218, 16777219, -16777217,
                                (long long)0x7fffffffffffffffull, (long long)0x8000000000000000ull,
                                (1ll << 62) + (1ll << 38), (1ll << 62) + (1ll << 38) + 1, -((1ll << 40) + (1ll << 16))};
    for (long long v : ledges) check_l(v);
    for (int i = 0; i < 4000000; i++) {
        const unsigned long long r = rng();
        const int sh = (int)(rng() % 64);
        check_l((long long)r);
        check_l((long long)(r >> sh));
        check_l(-(long long)(r >> (sh | 1)));
    }
    std::printf("%ld %ld\n", checked, bad);
    return bad != 0;
}
'''


def test_integer_conversions_match_round_to_nearest_even(tmp_path):
    src = tmp_path / "fp.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "fp"
    inc = os.path.join(ROOT, "openbcsim_gb300", "csrc")
    out = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{inc}", str(src), "-o", str(exe)],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr[-3000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    checked, bad = map(int, run.stdout.split()[-2:])
    assert bad == 0 and checked > 10_000_000
