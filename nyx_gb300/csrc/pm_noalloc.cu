// nyxpm_deposit_noalloc: the CIC mass density of particles that are already in
// device memory, computed without allocating any device memory.
//
// Who needs it: a host code whose device memory is owned by its own arena
// allocator (an AMReX build reserves most of the GPU in its arena at start-up
// and hands out pieces of it) cannot let a library call cudaMalloc behind its
// back -- the call can fail for lack of free memory or fragment the memory the
// arena manages.  Such a caller passes its own input and output buffers; the
// scratch the counting sort needs lives in a file-scope __device__ array that
// every GPU which loads this library holds until the process exits.
//
// Limits: grid edge n <= 64 (262,144 cells) and at most 262,144 particles, so
// the array is ~10 MiB.  Larger problems go through nyxpm_box_create /
// nyxpm_deposit, which allocate.
//
// The arithmetic (key, sort order, per-key partial sums, cell sums) is that of
// nyxpm_deposit for uniform masses, so both give the same density bit for bit.
// Like nyxpm_deposit it refuses non-finite positions: the key pass counts them,
// and the call reads the count back before it returns.
// Built with --fmad=false like the other FP64 units.
#include "pm_common.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace nyxpm {

namespace {

constexpr int kNaMaxN = 64;
constexpr long long kNaMaxCells = (long long)kNaMaxN * kNaMaxN * kNaMaxN;
constexpr long long kNaMaxParticles = 262144;
constexpr int kNaScanT = 512, kNaScanIPT = 8, kNaScanTile = kNaScanT * kNaScanIPT;
constexpr long long kNaTiles = (kNaMaxCells + kNaScanTile - 1) / kNaScanTile;

// scratch layout, each part rounded up to 256 bytes
constexpr size_t up256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr size_t kOffCount = 0;
constexpr size_t kOffStart = kOffCount + up256(4 * kNaMaxCells);
constexpr size_t kOffTiles = kOffStart + up256(4 * (kNaMaxCells + 1));
constexpr size_t kOffLongCount = kOffTiles + up256(4 * (kNaTiles + 1));
constexpr size_t kOffLongList = kOffLongCount + 256;
constexpr size_t kOffKey = kOffLongList + up256(4 * (kNaMaxParticles / 32 + 2));
constexpr size_t kOffPerm = kOffKey + up256(4 * kNaMaxParticles);
constexpr size_t kOffX = kOffPerm + up256(4 * kNaMaxParticles);
constexpr size_t kOffY = kOffX + up256(8 * kNaMaxParticles);
constexpr size_t kOffZ = kOffY + up256(8 * kNaMaxParticles);
constexpr size_t kScratchBytes = kOffZ + up256(8 * kNaMaxParticles);

// the scratch: every call shares it, and it keeps the last call's contents
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {};
int g_sm_count[kMaxDevices] = {};

// The device address of the scratch on the current device (the host-side name
// of the array is not a device address).  It is looked up again on every call
// whose stream is not capturing -- a device reset reloads the module and may
// move the array -- and the last address found is used while a capture runs.
nyxpm_status scratch_address(cudaStream_t stream, unsigned char** out, int* sm_count, bool* capturing,
                             char* errbuf, size_t errlen)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        if (errbuf && errlen) std::snprintf(errbuf, errlen, "no current CUDA device");
        return NYXPM_NO_DEVICE;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusNone;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev] || cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            if (errbuf && errlen)
                std::snprintf(errbuf, errlen, "cudaGetSymbolAddress of the scratch failed: %s",
                              cudaGetErrorString(e));
            return NYXPM_CUDA_ERROR;
        }
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            sms = 1;
        }
        g_sm_count[dev] = sms > 0 ? sms : 1;
    }
    *out = g_scratch_addr[dev];
    *sm_count = g_sm_count[dev];
    *capturing = cap != cudaStreamCaptureStatusNone;
    return NYXPM_OK;
}

__device__ __forceinline__ int na_key1(double x, double dxi, int n, double* frac)
{
    const double l = fma(x, dxi, 0.5);
    int il;
    const double fl = floor_int(l, &il);
    *frac = l - fl;
    return wrapi(il, n);
}

__global__ void na_zero(int* a, long long cnt)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cnt) a[t] = 0;
}

// A non-finite coordinate is counted in *bad (the call then refuses the input);
// its key is still a valid cell (the float-to-int conversion saturates and a NaN
// converts to 0), so no access leaves the arrays.
__global__ void na_keys(long long np, int n, double dxi, const double* __restrict__ x,
                        const double* __restrict__ y, const double* __restrict__ z, int* key, int* count,
                        int* bad)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const double px = x[q], py = y[q], pz = z[q];
    if (!(isfinite(px) && isfinite(py) && isfinite(pz))) atomicAdd(bad, 1);
    double f;
    const int i = na_key1(px, dxi, n, &f);
    const int j = na_key1(py, dxi, n, &f);
    const int k = na_key1(pz, dxi, n, &f);
    const int K = (int)cidx(i, j, k, n);
    key[q] = K;
    atomicAdd(count + K, 1);
}

__device__ __forceinline__ int na_warp_scan(int v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

__device__ int na_block_scan(int v, int* total)
{
    __shared__ int ws[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int inc = na_warp_scan(v);
    if (lane == 31) ws[w] = inc;
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        int s = lane < nw ? ws[lane] : 0;
        s = na_warp_scan(s);
        ws[lane] = s;
    }
    __syncthreads();
    const int before = (w > 0 ? ws[w - 1] : 0) + inc - v;
    *total = ws[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before;
}

__global__ void na_scan_reduce(const int* __restrict__ in, int cnt, int* tiles)
{
    const long long base = (long long)blockIdx.x * kNaScanTile + (long long)threadIdx.x * kNaScanIPT;
    int s = 0;
#pragma unroll
    for (int t = 0; t < kNaScanIPT; ++t)
        if (base + t < cnt) s += in[base + t];
    int total;
    na_block_scan(s, &total);
    if (threadIdx.x == 0) tiles[blockIdx.x] = total;
}

__global__ void na_scan_top(int* tiles, int ntiles)
{
    int carry = 0;
    for (int b0 = 0; b0 < ntiles; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        const int v = i < ntiles ? tiles[i] : 0;
        int total;
        const int ex = na_block_scan(v, &total);
        if (i < ntiles) tiles[i] = carry + ex;
        carry += total;
    }
}

__global__ void na_scan_down(const int* __restrict__ in, int cnt, const int* __restrict__ tiles, int* out)
{
    const long long base = (long long)blockIdx.x * kNaScanTile + (long long)threadIdx.x * kNaScanIPT;
    int v[kNaScanIPT];
    int s = 0;
#pragma unroll
    for (int t = 0; t < kNaScanIPT; ++t) {
        v[t] = base + t < cnt ? in[base + t] : 0;
        s += v[t];
    }
    int total;
    int run = na_block_scan(s, &total) + tiles[blockIdx.x];
#pragma unroll
    for (int t = 0; t < kNaScanIPT; ++t) {
        if (base + t < cnt) out[base + t] = run;
        run += v[t];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[cnt] = run;
}

__global__ void na_scatter(long long np, const int* __restrict__ key, const int* __restrict__ start,
                           int* count, int* perm)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int K = key[q];
    perm[start[K] + atomicSub(count + K, 1) - 1] = (int)q;
}

// order each key segment by original particle index (so the deposit order, and
// with it the density, does not depend on how the atomics were served)
__global__ void na_fix_short(int nc, const int* __restrict__ start, int* perm, int* long_list,
                             int* long_count)
{
    const int K = blockIdx.x * blockDim.x + threadIdx.x;
    if (K >= nc) return;
    const int s = start[K], len = start[K + 1] - s;
    if (len <= 1) return;
    if (len > 32) {
        long_list[atomicAdd(long_count, 1)] = K;
        return;
    }
    sort_short_segment(perm, s, len);
}

// Long segments: a rank sort by one block per segment (the values are distinct).
// A segment of up to kNaLongSmem entries is ranked from shared memory; a longer
// one (every particle in a few cells) from global memory.
constexpr int kNaLongSmem = 12288;

__global__ void na_fix_long(const int* __restrict__ start, const int* __restrict__ long_list,
                            const int* __restrict__ long_count, int* perm, int* tmp)
{
    __shared__ int sv[kNaLongSmem];
    const int total = *long_count;
    for (int li = blockIdx.x; li < total; li += gridDim.x) {
        const int K = long_list[li];
        const int s = start[K], len = start[K + 1] - s;
        const bool in_smem = len <= kNaLongSmem;
        __syncthreads();
        if (in_smem)
            for (int t = threadIdx.x; t < len; t += blockDim.x) sv[t] = perm[s + t];
        __syncthreads();
        for (int t = threadIdx.x; t < len; t += blockDim.x) {
            const int v = in_smem ? sv[t] : perm[s + t];
            int rank = 0;
            if (in_smem) {
                for (int u = 0; u < len; ++u) rank += sv[u] < v;
            } else {
                for (int u = 0; u < len; ++u) rank += perm[s + u] < v;
            }
            tmp[s + rank] = v;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < len; t += blockDim.x) perm[s + t] = tmp[s + t];
    }
}

__global__ void na_gather(long long np, const int* __restrict__ perm, const double* __restrict__ x,
                          const double* __restrict__ y, const double* __restrict__ z, double* xs,
                          double* ys, double* zs)
{
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= np) return;
    const int q = perm[s];
    xs[s] = x[q];
    ys[s] = y[q];
    zs[s] = z[q];
}

constexpr int kTx = 8, kTy = 8, kTz = 8;
constexpr int kKx = kTx + 1, kKy = kTy + 1, kKz = kTz + 1;
constexpr int kNKeys = kKx * kKy * kKz;

__device__ __forceinline__ void na_add_weights(int q, int n, double dxi,
                                               const double* __restrict__ x,
                                               const double* __restrict__ y,
                                               const double* __restrict__ z, double s[8])
{
    double fx, fy, fz;
    na_key1(x[q], dxi, n, &fx);
    na_key1(y[q], dxi, n, &fy);
    na_key1(z[q], dxi, n, &fz);
    const double sx[2] = {1.0 - fx, fx};
    const double sy[2] = {1.0 - fy, fy};
    const double sz[2] = {1.0 - fz, fz};
#pragma unroll
    for (int cz = 0; cz < 2; ++cz)
#pragma unroll
        for (int cy = 0; cy < 2; ++cy)
#pragma unroll
            for (int cx = 0; cx < 2; ++cx)
                s[cx + 2 * cy + 4 * cz] = s[cx + 2 * cy + 4 * cz] + (sx[cx] * sy[cy]) * sz[cz];
}

// A key longer than a warp, summed in the order the allocating deposit sums it
// with a whole warp: 32 lane partials (lane l: particles l, l+32, ... in order)
// combined by the xor butterfly 16, 8, 4, 2, 1.  Here one thread does it: the
// butterfly's result is the pairwise tree over the lanes taken in bit-reversed
// order, built with a stack of finished subtrees (a binary counter).
__device__ void na_long_key(int b0, int e, int n, double dxi, const double* __restrict__ x,
                            const double* __restrict__ y, const double* __restrict__ z,
                            double out[8])
{
    double stack[6][8];
    int depth = 0;
    for (int t = 0; t < 32; ++t) {
        const int lane = (int)(__brev((unsigned)t) >> 27);
        double* p = stack[depth++];
        for (int c = 0; c < 8; ++c) p[c] = 0.0;
        for (int q = b0 + lane; q < e; q += 32) na_add_weights(q, n, dxi, x, y, z, p);
        for (int v = t + 1; (v & 1) == 0; v >>= 1) {
            for (int c = 0; c < 8; ++c) stack[depth - 2][c] = stack[depth - 2][c] + stack[depth - 1][c];
            --depth;
        }
    }
    for (int c = 0; c < 8; ++c) out[c] = stack[0][c];
}

// per-key partial sums of the 8 corner weights, then cell sums in a fixed order
__global__ void __launch_bounds__(256) na_deposit(int n, double dxi, double scale,
                                                  const double* __restrict__ x,
                                                  const double* __restrict__ y,
                                                  const double* __restrict__ z,
                                                  const int* __restrict__ start, double* rho)
{
    __shared__ double part[kNKeys * 8];
    const int i0 = blockIdx.x * kTx, j0 = blockIdx.y * kTy, k0 = blockIdx.z * kTz;
    for (int kl = threadIdx.x; kl < kNKeys; kl += blockDim.x) {
        const int ki = kl % kKx, kj = (kl / kKx) % kKy, kk = kl / (kKx * kKy);
        const long long K = cidx(wrapi(i0 + ki, n), wrapi(j0 + kj, n), wrapi(k0 + kk, n), n);
        double s[8];
        const int b0 = start[K], e = start[K + 1];
        if (e - b0 > 32) {
            na_long_key(b0, e, n, dxi, x, y, z, s);
        } else {
#pragma unroll
            for (int c = 0; c < 8; ++c) s[c] = 0.0;
            for (int q = b0; q < e; ++q) na_add_weights(q, n, dxi, x, y, z, s);
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) part[kl * 8 + c] = s[c];
    }
    __syncthreads();
    for (int cl = threadIdx.x; cl < kTx * kTy * kTz; cl += blockDim.x) {
        const int ci = cl % kTx, cj = (cl / kTx) % kTy, ck = cl / (kTx * kTy);
        const int i = i0 + ci, j = j0 + cj, k = k0 + ck;
        if (i >= n || j >= n || k >= n) continue;
        double acc = 0.0;
#pragma unroll
        for (int dk = 0; dk < 2; ++dk)
#pragma unroll
            for (int dj = 0; dj < 2; ++dj)
#pragma unroll
                for (int di = 0; di < 2; ++di) {
                    const int kl = (ci + di) + kKx * ((cj + dj) + kKy * (ck + dk));
                    acc = acc + part[kl * 8 + (1 - di) + 2 * (1 - dj) + 4 * (1 - dk)];
                }
        rho[cidx(i, j, k, n)] = acc * scale;
    }
}

}  // namespace

}  // namespace nyxpm

using namespace nyxpm;

extern "C" nyxpm_status nyxpm_deposit_noalloc(const double* d_x, const double* d_y, const double* d_z,
                                              int64_t np, double mass, int n, double L, double* d_rho,
                                              void* stream, char* errbuf, size_t errlen)
{
    if (errbuf && errlen) errbuf[0] = '\0';
    auto fail = [&](nyxpm_status st, const char* msg) {
        if (errbuf && errlen) std::snprintf(errbuf, errlen, "%s", msg);
        return st;
    };
    if (!d_x || !d_y || !d_z || !d_rho) return fail(NYXPM_INVALID_ARG, "null device pointer");
    if (n < 1 || n > kNaMaxN)
        return fail(NYXPM_INVALID_ARG, "grid edge n must be in [1, 64] (the no-allocation scratch limit)");
    if (np < 1 || np > kNaMaxParticles)
        return fail(NYXPM_INVALID_ARG,
                    "particle count must be in [1, 262144] (the no-allocation scratch limit)");
    if (!(L > 0) || !std::isfinite(L)) return fail(NYXPM_INVALID_ARG, "box length must be positive");
    if (!(mass >= 0) || !std::isfinite(mass)) return fail(NYXPM_INVALID_ARG, "mass must be finite, >= 0");
    unsigned char* base = nullptr;
    int sm_count = 1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    bool capturing = false;
    const nyxpm_status st = scratch_address(s, &base, &sm_count, &capturing, errbuf, errlen);
    if (st != NYXPM_OK) return st;
    int* count = reinterpret_cast<int*>(base + kOffCount);
    int* start = reinterpret_cast<int*>(base + kOffStart);
    int* tiles = reinterpret_cast<int*>(base + kOffTiles);
    int* long_count = reinterpret_cast<int*>(base + kOffLongCount);
    int* bad = long_count + 1;   // non-finite positions seen
    int* long_list = reinterpret_cast<int*>(base + kOffLongList);
    int* key = reinterpret_cast<int*>(base + kOffKey);
    int* perm = reinterpret_cast<int*>(base + kOffPerm);
    double* xs = reinterpret_cast<double*>(base + kOffX);
    double* ys = reinterpret_cast<double*>(base + kOffY);
    double* zs = reinterpret_cast<double*>(base + kOffZ);
    const int nc = n * n * n;
    const double dxi = (double)n / L;
    const double dx = L / n;
    const double scale = mass * (1.0 / (dx * dx * dx));
    const unsigned pb = (unsigned)((np + 255) / 256);
    const unsigned cb = (unsigned)((nc + 255) / 256);
    const int ntiles = (nc + kNaScanTile - 1) / kNaScanTile;
    // the counts, the long-segment counter and the non-finite count must start at
    // zero: the array keeps whatever the previous call (or an interrupted one) left
    na_zero<<<cb, 256, 0, s>>>(count, nc);
    na_zero<<<1, 32, 0, s>>>(long_count, 2);
    na_keys<<<pb, 256, 0, s>>>(np, n, dxi, d_x, d_y, d_z, key, count, bad);
    na_scan_reduce<<<ntiles, kNaScanT, 0, s>>>(count, nc, tiles);
    na_scan_top<<<1, 1024, 0, s>>>(tiles, ntiles);
    na_scan_down<<<ntiles, kNaScanT, 0, s>>>(count, nc, tiles, start);
    na_scatter<<<pb, 256, 0, s>>>(np, key, start, count, perm);
    na_fix_short<<<cb, 256, 0, s>>>(nc, start, perm, long_list, long_count);
    na_fix_long<<<2 * sm_count, 512, 0, s>>>(start, long_list, long_count, perm, key);
    na_gather<<<pb, 256, 0, s>>>(np, perm, d_x, d_y, d_z, xs, ys, zs);
    const dim3 grid((n + kTx - 1) / kTx, (n + kTy - 1) / kTy, (n + kTz - 1) / kTz);
    na_deposit<<<grid, 256, 0, s>>>(n, dxi, scale, xs, ys, zs, start, d_rho);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        if (errbuf && errlen) std::snprintf(errbuf, errlen, "kernel launch failed: %s", cudaGetErrorString(e));
        return NYXPM_CUDA_ERROR;
    }
    // refuse non-finite positions as nyxpm_deposit does: read the count back
    // (into a host variable, no allocation), which waits for the stream.  A
    // stream under capture cannot be waited for: the graph holds the deposit
    // alone, and the check is the caller's (every replay's positions finite).
    if (capturing) return NYXPM_OK;
    int h_bad = 0;
    const cudaError_t ec = cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    const cudaError_t es = ec == cudaSuccess ? cudaStreamSynchronize(s) : ec;
    if (es != cudaSuccess) {
        cudaGetLastError();
        if (errbuf && errlen) std::snprintf(errbuf, errlen, "deposit failed: %s", cudaGetErrorString(es));
        return NYXPM_CUDA_ERROR;
    }
    if (h_bad != 0)
        return fail(NYXPM_INVALID_ARG, "non-finite particle position (rho holds no valid density)");
    return NYXPM_OK;
}
