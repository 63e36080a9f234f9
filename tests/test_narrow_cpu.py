"""The update kernels write the FP32 mirror of the state with an FP64 -> FP32 rounding done on the
integer pipes (f64_bits_to_f32_bits in hos_f32x2.cuh), in place of the conversion instruction that
runs on GB300's narrow FP64 pipe.  The mirror must hold the same values float(x) gives, since the
TMA-staged FP32 face kernels read it where the converting FP32 kernels round the FP64 state
themselves.  This test compiles the routine for the host and compares it with the host's IEEE
round-to-nearest-even conversion (FP32 subnormal results flushed to signed zero, as the -ftz build
flushes them) on random bit patterns, on every exponent around FP32's range with ties and
near-ties of the dropped bits, and on zeros, infinities and NaN."""
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "high-order-solver_gb300" / "csrc"

PROGRAM = r"""
#include "hos_f32x2.cuh"
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
static unsigned expect(double x) {
    const float f = (float)x;
    unsigned u;
    std::memcpy(&u, &f, 4);
    if (std::isnan(f)) return 0x7fffffffu;
    if ((u & 0x7f800000u) == 0u) return u & 0x80000000u;   // subnormal: signed zero
    return u;
}
static unsigned got(double x) {
    std::uint64_t b;
    std::memcpy(&b, &x, 8);
    return hos::f64_bits_to_f32_bits((unsigned)(b >> 32), (unsigned)b);
}
int main() {
    std::mt19937_64 g(20261204);
    long long n = 0, bad = 0;
    auto check = [&](double x) {
        ++n;
        if (expect(x) != got(x) && bad++ < 5) std::printf("%a: %08x != %08x\n", x, got(x), expect(x));
    };
    for (int i = 0; i < 4000000; ++i) {
        const std::uint64_t b = g();
        double x;
        std::memcpy(&x, &b, 8);
        check(x);
    }
    for (int e = 850; e <= 1170; ++e)
        for (int k = 0; k < 20000; ++k) {
            std::uint64_t m = g() & ((1ull << 52) - 1);
            const std::uint64_t low = (1ull << 29) - 1;
            if (k % 4 == 1) m = (m & ~low) | (1ull << 28);         // a tie
            if (k % 4 == 2) m = (m & ~low) | ((1ull << 28) - 1);   // just below a tie
            if (k % 4 == 3) m |= low;                               // just below the next value
            if (k == 0) m = (1ull << 52) - 1;
            const std::uint64_t b = ((std::uint64_t)e << 52) | m | ((g() & 1) << 63);
            double x;
            std::memcpy(&x, &b, 8);
            check(x);
        }
    const double special[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 1.0, 0.1, 1.4, 0.5323, -1.206,
                              3.4028234663852886e38, 3.4028235677973366e38, 1e39, -1e300,
                              1.1754943508222875e-38, 1.1754942807573643e-38, 1e-45, 1e-300};
    for (double x : special) check(x);
    std::printf("%lld %lld\n", n, bad);
    return bad != 0;
}
"""


def test_integer_pipe_narrowing_equals_ieee_rounding(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if Path("/usr/local/cuda/bin/nvcc").exists() else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    src = tmp_path / "narrow.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "narrow"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", f"-I{CSRC}",
                    "-o", str(exe), str(src)], check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    n, bad = map(int, r.stdout.split()[-2:])
    assert bad == 0 and n > 10_000_000


def test_speed_bit_patterns_order_as_doubles():
    """The update kernels take the block's largest CFL signal speed on the speeds' bit patterns
    read as signed 64-bit integers (reduce_block_speed in hos_step.cuh): a speed is -1 (a cell with
    no candidate), +0 (a speed that was not finite) or a positive finite double, and over those
    values the integer order must be the double order."""
    import numpy as np

    rng = np.random.default_rng(7)
    pos = np.concatenate([rng.uniform(0.0, 10.0, 20000), 10.0 ** rng.uniform(-300, 300, 20000),
                          [np.finfo(np.float64).tiny, 5e-324, np.finfo(np.float64).max, 1.0]])
    vals = np.concatenate([[-1.0, 0.0], pos[pos > 0]])
    bits = vals.view(np.int64)
    order_d = np.argsort(vals, kind="stable")
    order_i = np.argsort(bits, kind="stable")
    assert np.array_equal(vals[order_d], vals[order_i])
    # and the maximum of any subset agrees
    for _ in range(200):
        sub = rng.choice(vals.size, 256)
        assert vals[sub].max() == vals[sub][np.argmax(bits[sub])]
