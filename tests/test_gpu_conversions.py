"""The FP64 <-> FP32 conversions on the integer pipes (f64_to_f32_rn and
f32_to_f64, nyx_gb300/csrc/pm_common.cuh), the integer floor (floor_int) and the
integer-compare periodic wrap (wrap_pos) against the hardware operations, bit
for bit (tolerance: exact), on the GPU.

The mixed-precision kernels use them in place of the conversion instructions,
which run on GB300's FP64 pipe; their results must not change.  A probe compiled
here with nvcc for sm_103a compares:
* float -> double: all 2^32 float bit patterns;
* double -> float: 2^28 bit patterns from a hash of the index (every exponent),
  and, for every exponent from 2^-150 to 2^130 and both signs, the fraction
  patterns at the rounding boundaries (dropped bits 0, 1, just below, at and
  just above one half, all ones; kept bits even, odd, all ones: ties to even,
  carries into the exponent, overflow to infinity, the subnormal edge), plus
  zeros, subnormals, infinities and NaNs;
* floor_int against floor and (int)floor: 2^26 hashed doubles in (-1, 1100) and
  2^26 hashed bit patterns of either sign between 2^-24 and 2^36, and the
  edges (-1, just above -1, -0.0, +0.0, subnormals, 2^31 - 1, 2^31, NaN, inf);
* wrap_pos against the floating-point comparisons: 2^26 values in [-2L, 2L) for
  L = 1, 7.5 and 0.3, and the edges (L, the double below L, -0.0, +0.0, -tiny,
  2L, -L, NaN, +-inf).
"""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
#include <cstdio>
#include <cstdint>
#include "pm_common.cuh"
using namespace nyxpm;

__device__ unsigned long long g_bad[6];
__device__ unsigned long long g_first[2];

__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__device__ void check_d2f(unsigned long long bits, int slot)
{
    const double x = __longlong_as_double((long long)bits);
    const unsigned a = __float_as_uint(f64_to_f32_rn(x)), b = __float_as_uint((float)x);
    if (a != b) {
        if (atomicAdd(&g_bad[slot], 1ULL) == 0ULL) g_first[0] = bits;
    }
}

__global__ void k_f2d(unsigned long long total)
{
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const float f = __uint_as_float((unsigned)i);
        const unsigned long long a = (unsigned long long)__double_as_longlong(f32_to_f64(f));
        const unsigned long long b = (unsigned long long)__double_as_longlong((double)f);
        if (a != b) {
            if (atomicAdd(&g_bad[0], 1ULL) == 0ULL) g_first[1] = i;
        }
    }
}

__global__ void k_d2f_random(unsigned long long total)
{
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x)
        check_d2f(mix64(i), 1);
}

// exponent e (biased, 874 .. 1153), sign, 6 dropped-bit patterns x 5 kept-bit patterns
__global__ void k_d2f_edges()
{
    const unsigned rest[6] = {0u, 1u, 0x0fffffffu, 0x10000000u, 0x10000001u, 0x1fffffffu};
    const unsigned kept[5] = {0u, 1u, 2u, 0x7ffffeu, 0x7fffffu};
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int e = 874 + t / 60, r = t % 60;
    if (e > 1153) return;
    const unsigned long long frac = ((unsigned long long)kept[(r / 6) % 5] << 29) | rest[r % 6];
    const unsigned long long sign = (r / 30) ? 0x8000000000000000ULL : 0ULL;
    check_d2f(sign | ((unsigned long long)e << 52) | frac, 2);
}

__global__ void k_d2f_specials()
{
    const unsigned long long v[12] = {0ULL, 0x8000000000000000ULL, 1ULL, 0x000fffffffffffffULL,
                                      0x7ff0000000000000ULL, 0xfff0000000000000ULL,
                                      0x7ff8000000000000ULL, 0x7ff0000000000001ULL,
                                      0x7fefffffffffffffULL, 0x47efffffe0000000ULL,
                                      0x47effffff0000000ULL, 0x3810000000000000ULL};
    if (threadIdx.x < 12) check_d2f(v[threadIdx.x], 3);
}

// floor_int against floor and (int)floor: hashed doubles in (-1, 1100), hashed
// bit patterns with exponents 2^-24 .. 2^36 and either sign, and the edges
__device__ void check_floor(double l)
{
    int ia = 0;
    const double fa = floor_int(l, &ia);
    const double fb = floor(l);
    const int ib = (int)fb;
    if (__double_as_longlong(fa) != __double_as_longlong(fb) || ia != ib) atomicAdd(&g_bad[4], 1ULL);
}

__global__ void k_floor(unsigned long long total)
{
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long u = mix64(i ^ 0x5bd1e995ULL);
        check_floor((double)(u >> 11) * 0x1.0p-53 * 1101.0 - 1.0);
        const unsigned long long e = 1023ULL - 24ULL + (u % 61ULL);
        check_floor(__longlong_as_double((long long)((u & 0x800fffffffffffffULL) | (e << 52))));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const double edges[16] = {-1.0, -1.0 + 0x1.0p-53, -0x1.0p-1074, -0.0, 0.0, 0.5, 1.0,
                                  1.0 - 0x1.0p-53, 2147483647.0, 2147483647.5, 2147483648.0,
                                  -2.5, 1e300, __longlong_as_double(0x7ff8000000000000LL),
                                  __longlong_as_double(0x7ff0000000000000LL), 0x1.0p-1074};
        for (int t = 0; t < 16; ++t) check_floor(edges[t]);
    }
}

// wrap_pos against the floating-point comparisons, for boxes of side 1, 7.5 and 0.3
__device__ void check_wrap(double v, double L)
{
    const double a = wrap_pos(v, L), b = wrap_pos_hw(v, L);
    if (__double_as_longlong(a) != __double_as_longlong(b)) atomicAdd(&g_bad[5], 1ULL);
}

__global__ void k_wrap(unsigned long long total)
{
    const double Ls[3] = {1.0, 7.5, 0.3};
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long u = mix64(i ^ 0x9e3779b9ULL);
        const double L = Ls[u % 3];
        check_wrap(((double)(u >> 11) * 0x1.0p-53 * 4.0 - 2.0) * L, L);
    }
    if (blockIdx.x == 0 && threadIdx.x < 3) {
        const double L = Ls[threadIdx.x];
        const double lm = __longlong_as_double(__double_as_longlong(L) - 1);
        const double edges[12] = {L, lm, -0.0, 0.0, -0x1.0p-1074, -0x1.0p-60, 2.0 * L, -L,
                                  __longlong_as_double(0x7ff8000000000000LL),
                                  __longlong_as_double(0x7ff0000000000000LL),
                                  __longlong_as_double((long long)0xfff0000000000000ULL), -2.0 * L};
        for (int t = 0; t < 12; ++t) check_wrap(edges[t], L);
    }
}

int main()
{
    k_f2d<<<152 * 8, 256>>>(1ULL << 32);
    k_d2f_random<<<152 * 8, 256>>>(1ULL << 28);
    k_d2f_edges<<<(280 * 60 + 255) / 256, 256>>>();
    k_d2f_specials<<<1, 32>>>();
    k_floor<<<152 * 8, 256>>>(1ULL << 26);
    k_wrap<<<152 * 8, 256>>>(1ULL << 26);
    if (cudaDeviceSynchronize() != cudaSuccess) { printf("cuda error\n"); return 2; }
    unsigned long long bad[6], first[2];
    cudaMemcpyFromSymbol(bad, g_bad, sizeof(bad));
    cudaMemcpyFromSymbol(first, g_first, sizeof(first));
    printf("f2d %llu d2f_random %llu d2f_edges %llu d2f_specials %llu floor %llu wrap %llu first %016llx %08llx\n",
           bad[0], bad[1], bad[2], bad[3], bad[4], bad[5], first[0], first[1]);
    return 0;
}
"""


@pytest.mark.skipif(not gpu_available(), reason="no GPU")
@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="no nvcc")
def test_integer_pipe_conversions_equal_the_hardware(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "conv.cu"
    src.write_text(PROBE)
    exe = tmp_path / "conv"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "--expt-relaxed-constexpr", "-I", os.path.join(REPO, "nyx_gb300", "csrc"),
                    "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=300).stdout
    words = out.split()
    counts = {words[i]: int(words[i + 1]) for i in range(0, 12, 2)}
    assert counts == {"f2d": 0, "d2f_random": 0, "d2f_edges": 0, "d2f_specials": 0, "floor": 0,
                      "wrap": 0}, out
