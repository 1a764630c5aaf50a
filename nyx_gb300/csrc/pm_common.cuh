// Internal declarations shared by the translation units of libnyxpm.
//
// Layouts in device memory (one box = one periodic n^3 grid):
//   particles  structure of arrays, FP64: x y z vx vy vz [m] id, kept sorted by
//              deposit key (cell of floor(x/dx + 1/2)), double-buffered for the
//              counting-sort gather;
//   cell index c = i + n*(j + n*k), x fastest;
//   rho        n^3, natural layout;
//   multigrid  every smoothed level stores phi and rhs red-black split: the red
//              cells ((i+j+k) even) and the black cells in two arrays of n^3/2,
//              compact index (i>>1) + (n/2)*(j + n*k), so a half sweep streams
//              exactly one array of each colour; the coarsest level (n <= 8) is
//              natural layout.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "../../include/nyxpm.h"

namespace nyxpm {

constexpr int kMaxBottom = 8;          // largest coarsest-grid edge (solved exactly)
// A deposit key with more particles than this is summed by a whole warp in
// lane-strided partials (lane l: particles l, l+32, ...) and an xor butterfly;
// shorter keys are summed in order by one thread.  The sort queues exactly
// these keys (segments longer than a warp) in long_list.
constexpr int kDepositLanes = 32;
constexpr int kCoarsenAbove = 4;       // levels halve while the edge is even and above this

// |v| as ordered bits: for non-negative doubles the bit patterns order like the
// values and a NaN orders above every number, so max reductions run on the
// integer pipe (FP64 compares would take FP64 issue slots)
// Conversions between FP64 and FP32 on the integer pipes.  On GB300 the FP64
// pipe issues at a small fraction of the FP32 rate, and the hardware conversion
// instructions between the two formats run on it; the FP32 kernels of the mixed
// form that round FP64 values to FP32 use these instead.  Both follow IEEE 754
// directly: a double whose float rounding is a normal float (exponent
// -126 .. 127) keeps its sign, its exponent rebiased (1023 -> 127) and the top 23
// of its 52 fraction bits, and the 29 dropped bits round to nearest, ties to
// even (a carry out of the fraction steps the exponent, up to infinity, as the
// rounding demands).  Zeros, values that round into the float subnormal range,
// and infinities and NaNs go to the hardware conversion.  The results are the
// hardware's, bit for bit.  The hardware paths are calls, not inlined, so that
// the compiler branches around them instead of converting every value and
// selecting.
static __device__ __noinline__ float f64_to_f32_hw(double x) { return (float)x; }
static __device__ __noinline__ double f32_to_f64_hw(float f) { return (double)f; }

__device__ __forceinline__ float f64_to_f32_rn(double x)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
    const unsigned e = (hi >> 20) & 0x7ffu;                // biased FP64 exponent
    if (e - 897u > 253u) return f64_to_f32_hw(x);           // outside 2^-126 .. 2^127
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 fraction bits
    const unsigned rest = lo & 0x1fffffffu;                  // the 29 dropped bits
    unsigned bits = (hi & 0x80000000u) | ((e - 896u) << 23) | m;
    bits += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return __uint_as_float(bits);
}

// a normal float, exactly, as a double (zeros, subnormals, infinities and NaNs:
// the hardware conversion)
__device__ __forceinline__ double f32_to_f64(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned ef = (b >> 23) & 0xffu;
    if (ef - 1u > 253u) return f32_to_f64_hw(f);
    const unsigned hi = (b & 0x80000000u) | ((ef + 896u) << 20) | ((b & 0x7fffffu) >> 3);
    const unsigned lo = b << 29;
    return __longlong_as_double((long long)(((unsigned long long)hi << 32) | lo));
}

// floor(l) as a double and as an int, on the integer pipes (floor and the
// double -> int conversion run on the FP64 pipe): for l in [0, 2^31) the
// fraction bits below the binary point are cleared; (-1, 0) gives -1 and -0.0
// gives -0.0, as floor does.  Anything else (l <= -1, l >= 2^31, NaN) goes to
// floor itself.  The same values as floor and (int)floor, bit for bit.
static __device__ __noinline__ double floor_hw(double l, int* i)
{
    const double f = floor(l);
    *i = (int)f;
    return f;
}

__device__ __forceinline__ double floor_int(double l, int* i)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(l);
    const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
    if ((u >> 63) == 0) {
        if (e < 1023u) {   // [+0, 1)
            *i = 0;
            return 0.0;
        }
        if (e < 1054u) {   // [1, 2^31): 1075 - e = 22 .. 52 fraction bits below the point
            const unsigned sh = 1075u - e;
            *i = (int)(((u & 0xfffffffffffffULL) | (1ULL << 52)) >> sh);
            return __longlong_as_double((long long)(u & (~0ULL << sh)));
        }
    } else if (e < 1023u) {   // (-1, -0]
        if ((u << 1) == 0) {
            *i = 0;
            return l;   // -0.0
        }
        *i = -1;
        return -1.0;
    }
    return floor_hw(l, i);
}

static __device__ __noinline__ double wrap_pos_hw(double v, double L)
{
    if (v >= L) v = v - L;
    else if (v < 0.0) v = v + L;
    if (v >= L) v = 0.0;
    return v;
}

// the periodic shift into [0, L) (L > 0).  For a finite v the comparisons are
// integer comparisons of the bit patterns (for L > 0, v >= L exactly when v's
// pattern, read as a signed integer, is not below L's; v < 0 when the sign bit
// is set and v is not -0.0), off the FP64 pipe; infinities and NaNs take the
// floating-point comparisons.  The same results, bit for bit.
__device__ __forceinline__ double wrap_pos(double v, double L)
{
    const long long bv = __double_as_longlong(v), bL = __double_as_longlong(L);
    const unsigned long long uv = (unsigned long long)bv;
    if (((uv >> 52) & 0x7ffULL) == 0x7ffULL) return wrap_pos_hw(v, L);
    if (bv >= bL) v = v - L;
    else if (bv < 0 && (uv << 1) != 0) v = v + L;
    if (__double_as_longlong(v) >= bL) v = 0.0;
    return v;
}

__host__ __device__ inline unsigned long long absbits(double v)
{
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
#else
    unsigned long long u;
    __builtin_memcpy(&u, &v, sizeof(u));
    return u & 0x7fffffffffffffffULL;
#endif
}

// block max of bits into *out (blocks are whole warps)
__device__ inline void block_umax_store(unsigned long long v, unsigned long long* out)
{
    __shared__ unsigned long long sm[32];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const unsigned long long o = __shfl_down_sync(0xffffffffu, v, off);
        v = o > v ? o : v;
    }
    const int lane = tid & 31, w = tid >> 5;
    if (lane == 0) sm[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (nthreads >> 5) ? sm[lane] : 0ULL;
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            const unsigned long long o = __shfl_down_sync(0xffffffffu, v, off);
            v = o > v ? o : v;
        }
        if (lane == 0) atomicMax(out, v);
    }
    __syncthreads();  // sm may be reused by the caller's next loop iteration
}

// warp max of bits into *out; the whole warp calls it (blocks of 32-wide rows)
// Sorts a[s .. s+len) ascending, 2 <= len <= 32, values distinct and below
// INT32_MAX: the counting sort's segment of one key, put back in particle order.
// Up to 4 values (most segments at a particle per cell) go through a sorting
// network in registers; longer ones through an insertion sort.
__device__ __forceinline__ void sort_short_segment(int* a, int s, int len)
{
    if (len <= 4) {
        int v0 = a[s], v1 = a[s + 1];
        int v2 = len > 2 ? a[s + 2] : INT32_MAX, v3 = len > 3 ? a[s + 3] : INT32_MAX;
        auto cs = [](int& x, int& y) {
            const int lo = min(x, y), hi = max(x, y);
            x = lo;
            y = hi;
        };
        cs(v0, v1);
        cs(v2, v3);
        cs(v0, v2);
        cs(v1, v3);
        cs(v1, v2);
        a[s] = v0;
        a[s + 1] = v1;
        if (len > 2) a[s + 2] = v2;
        if (len > 3) a[s + 3] = v3;
        return;
    }
    int v[32];
#pragma unroll
    for (int t = 0; t < 32; ++t)
        if (t < len) v[t] = a[s + t];
    for (int i = 1; i < len; ++i) {
        const int cur = v[i];
        int j = i - 1;
        while (j >= 0 && v[j] > cur) {
            v[j + 1] = v[j];
            --j;
        }
        v[j + 1] = cur;
    }
#pragma unroll
    for (int t = 0; t < 32; ++t)
        if (t < len) a[s + t] = v[t];
}

__device__ inline void warp_umax_atomic(unsigned long long v, unsigned long long* out)
{
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, v, off);
        v = o > v ? o : v;
    }
    const int lane = (threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z)) & 31;
    if (lane == 0 && v != 0ULL) atomicMax(out, v);
}

// One multigrid level.  The right-hand side is stored in smoother units,
// beta = h^2 rhs / 6, so a Gauss-Seidel update is phi = s/6 - beta (s = sum of
// the 6 neighbours) and the h factors of coarser levels are exact powers of 2.
struct Level {
    int n = 0;
    int split = 0;                     // 1: red/black arrays, 0: natural layout
    double* phi_r = nullptr;           // split: red n^3/2; natural: n^3
    double* phi_b = nullptr;           // split: black n^3/2; natural: unused
    double* beta_r = nullptr;
    double* beta_b = nullptr;
    // FP32 copies for the mixed-precision inner V-cycles
    float* fphi_r = nullptr;
    float* fphi_b = nullptr;
    float* fbeta_r = nullptr;
    float* fbeta_b = nullptr;
};

// device view of one level
struct LevelView {
    int n, split;
    double* phi_r;
    double* phi_b;
    double* beta_r;
    double* beta_b;
};

struct LevelViewF {
    int n, split;
    float* phi_r;
    float* phi_b;
    float* beta_r;
    float* beta_b;
};

inline LevelView view(const Level& l)
{
    return LevelView{l.n, l.split, l.phi_r, l.phi_b, l.beta_r, l.beta_b};
}

inline LevelViewF viewf(const Level& l)
{
    return LevelViewF{l.n, l.split, l.fphi_r, l.fphi_b, l.fbeta_r, l.fbeta_b};
}

// 3-D launch geometry without index division: x over the fastest index
// (rounded up to a power of two up to 32), y over rows, z over planes.
struct Geo {
    dim3 grid, block;
};

inline Geo geo3(int nx, int ny, int nz, int threads = 256)
{
    int bx = 1;
    while (bx < nx && bx < 32) bx <<= 1;
    int by = threads / bx;
    if (by > ny) {
        int p = 1;
        while (p < ny) p <<= 1;
        by = p;
    }
    if (bx * by < 32) by = 32 / bx;  // whole warps: the block reductions shuffle over 32 lanes
    Geo g;
    g.block = dim3(bx, by, 1);
    g.grid = dim3((nx + bx - 1) / bx, (ny + by - 1) / by, nz);
    return g;
}

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__host__ __device__ inline int wrapi(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

__host__ __device__ inline long long cidx(int i, int j, int k, int n)
{
    return (long long)i + (long long)n * ((long long)j + (long long)n * k);
}

// ---------------------------------------------------------------------------
// double-float (a pair hi + lo of FP32 numbers, |lo| <= ulp(hi)/2) arithmetic on
// the FP32 pipe, after Dekker (1971) and Knuth's TwoSum: the sum and product
// errors of FP32 operations are recovered exactly and carried in lo.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& err)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void df_fast_two_sum(float a, float b, float& s, float& err)
{
    // |a| >= |b| or a = 0
    s = __fadd_rn(a, b);
    err = __fsub_rn(b, __fsub_rn(s, a));
}

// A bound on the error df_residual_update adds to a tracked residual, per unit
// of max|e| over the cells it reads: the rounding of the six neighbour errors
// summed in FP32 (at most 150 * 2^-48), of the product by the two-word 1/6, of
// the subtraction of e and of the update of r (a few 2^-48 each).
constexpr double kDfUpdateErr = 160.0 / 281474976710656.0;   // 160 * 2^-48

// r -= L e at one cell, in double-float: L e = s/6 - e_m (smoother units), s the
// sum of the six neighbours v of the FP32 correction e, (c_hi, c_lo) = 1/6
__device__ __forceinline__ void df_residual_update(const float (&v)[6], float em, float c_hi,
                                                   float c_lo, float& rh, float& rl)
{
    float sh = v[0], sl = 0.f, err;
#pragma unroll
    for (int w = 1; w < 6; ++w) {
        df_two_sum(sh, v[w], sh, err);
        sl = __fadd_rn(sl, err);
    }
    const float ph = __fmul_rn(sh, c_hi);
    float pl = __fmaf_rn(sh, c_hi, -ph);
    pl = __fadd_rn(pl, __fadd_rn(__fmul_rn(sh, c_lo), __fmul_rn(sl, c_hi)));
    float dh;
    df_two_sum(ph, -em, dh, err);
    const float dl = __fadd_rn(pl, err);
    float uh;
    df_two_sum(rh, -dh, uh, err);
    const float ul = __fadd_rn(err, __fsub_rn(rl, dl));
    df_fast_two_sum(uh, ul, rh, rl);
}

// pointer to phi (or rhs) at cell (i,j,k) of a level in either layout
template <typename T>
__device__ inline T* lv_ptr(T* r, T* b, int n, int split, int i, int j, int k)
{
    if (!split) return r + cidx(i, j, k, n);
    const int half = n >> 1;
    T* base = ((i + j + k) & 1) ? b : r;
    return base + (long long)(i >> 1) + (long long)half * ((long long)j + (long long)n * k);
}

// ---------------------------------------------------------------------------
// box
// ---------------------------------------------------------------------------
struct ProfRec {
    int stage;
    int fine;
    double bytes;
};

struct Ctx;

// One solver iteration (V-cycle or defect-correction step, its residual norm and
// the norm's copy to the host) captured once per box and replayed: the launches
// of a box never change between solves, only the host reads the norm.
struct IterGraph {
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;              // kernel launches one replay stands for
    int failed = 0;                    // capture refused: enqueue eagerly from then on
};

struct Box {
    int n = 0;
    double L = 0, dx = 0, dxi = 0;
    int64_t np = 0;
    nyxpm_precision prec = NYXPM_FP64;
    int uniform_mass = 1;
    double mscalar = 0;
    double mass_offset = 0;
    int sorted = 0;
    int uploaded = 0;
    int have_phi = 0;
    int g_from_caller = 0;             // g (and g32) hold nyxpm_set_grav_vector's field

    // particles (FP64 form)
    double *x = nullptr, *y = nullptr, *z = nullptr, *vx = nullptr, *vy = nullptr, *vz = nullptr,
           *m = nullptr;
    int* id = nullptr;
    double *x2 = nullptr, *y2 = nullptr, *z2 = nullptr, *vx2 = nullptr, *vy2 = nullptr,
           *vz2 = nullptr, *m2 = nullptr;
    int* id2 = nullptr;

    // particles (mixed form): cell-relative FP32
    int* cell = nullptr;               // cell of floor(x/dx), packed i | j << 10 | k << 20
    float *ox = nullptr, *oy = nullptr, *oz = nullptr;   // offset within the cell, [0,1)
    float *fvx = nullptr, *fvy = nullptr, *fvz = nullptr;
    float* fm = nullptr;
    int* cell2 = nullptr;
    float *ox2 = nullptr, *oy2 = nullptr, *oz2 = nullptr, *fvx2 = nullptr, *fvy2 = nullptr,
          *fvz2 = nullptr, *fm2 = nullptr;

    // sort scratch
    int* key = nullptr;
    int* perm = nullptr;
    int* cell_count = nullptr;         // n^3, all zero between sorts
    int* cell_start = nullptr;         // n^3 + 1
    int* tile_sums = nullptr;
    int ntiles = 0;
    int* long_list = nullptr;          // keys of segments longer than a warp
    int* long_count = nullptr;
    // deposit partials of the keys in long_list (8 corners each), and the slot
    // of each such key (read only for keys longer than kDepositLanes)
    double* heavy_part = nullptr;
    int* key_slot = nullptr;
    double* key_part = nullptr;        // FP64: 8 n^3 per-key corner sums (two-pass deposit)

    // fields
    double* rho = nullptr;             // n^3
    float* frho = nullptr;             // n^3 (mixed)
    double* g = nullptr;               // 3 n^3, component-major, kept in step with phi
    double* nat = nullptr;             // n^3 natural-layout scratch for phi in/out
    double* rows = nullptr;            // n^2 row sums
    double* planes = nullptr;          // n plane sums
    double* scal = nullptr;            // [0] mean
    unsigned long long* norms = nullptr;   // [0] ||rhs||inf, [1] ||r||inf, [2] bad uploads,
                                           // [3] time-step limit, [4] mixed: max |e|
    unsigned long long* h_norms = nullptr; // pinned host mirror
    double* G = nullptr;               // bottom Green's function (smoother units)
    float* Gf = nullptr;               // the same in FP32 (mixed inner V-cycles)
    float* g32 = nullptr;              // mixed: FP32 gravity vector for the kicks, float4 per cell
    float* r_lo = nullptr;             // mixed: low words of the level-0 residual (red, black)
    double mscalar32_scale = 0;        // mixed: m / dx^3 applied to the FP32 deposit
    int nb = 0;
    std::vector<Level> levels;
    IterGraph iter_graph[4];           // solver iterations: [0] mixed / plain FP64; FP64 with
                                       // the fused norm: [opening 0 | later 2] + red array
    double* phi_r_alloc = nullptr;     // FP64: level 0's own red array
    double* phi_r_spare = nullptr;     // FP64: the other red array of level 0

    // host<->device staging: AoS pos (3 np), vel (3 np), mass (np) doubles
    double* staging = nullptr;

    std::vector<void*> allocs;
};

struct Ctx {
    nyxpm_params p{};
    cudaStream_t stream = nullptr;
    int own_stream = 0;
    std::string err;
    int64_t launches = 0;
    // profiling
    int prof_on = 0;
    std::vector<cudaEvent_t> ev_a, ev_b;
    std::vector<ProfRec> recs;
    nyxpm_profile acc{};
    int sm_count = 0;
    // second stream and events of the host-buffer step (created on first use)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copy_in = nullptr, ev_copy_out = nullptr;
    // multigrid kernels launched with programmatic dependent launch (off with
    // the environment variable NYXPM_NO_PDL set, for comparison)
    int pdl = 1;
    // the first error a launch_pdl returned since the last check_launch
    cudaError_t launch_error = cudaSuccess;
};

// Programmatic dependent launch: a kernel launched by launch_pdl may be scheduled
// while the kernel before it in the stream finishes its last blocks, hiding the
// launch gap between the short multigrid kernels (inside the solver graphs too).
// Every kernel launched this way starts with pdl_wait(), which returns once the
// previous kernel has completed and its writes are visible, before it reads or
// writes global memory; then pdl_trigger() lets the next kernel be scheduled once
// all of this kernel's blocks have started.  Launched without the attribute, both
// are no-ops, so the kernels are correct on every path.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline void launch_pdl(Ctx& c, void (*kernel)(KArgs...), dim3 grid, dim3 block, Args... args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = c.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = c.pdl ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
    if (e != cudaSuccess && c.launch_error == cudaSuccess) c.launch_error = e;   // check_launch reports it
}

// launch bookkeeping: call prof_begin before and prof_end after each launch
void prof_begin(Ctx& c);
void prof_end(Ctx& c, int stage, double bytes, int fine = 0);
nyxpm_status check_launch(Ctx& c, const char* what);
// Enqueue one solver iteration: eagerly while profiling (per-launch events), else
// by replaying the box's captured graph (captured on first use).
nyxpm_status run_iteration(Ctx& c, IterGraph& g, const std::function<nyxpm_status()>& body);

// ---------------------------------------------------------------------------
// launchers (defined in pm_particles.cu / pm_multigrid.cu / pm_mixed.cu)
// ---------------------------------------------------------------------------
nyxpm_status launch_unpack(Ctx& c, Box& b, const double* d_pos, const double* d_vel,
                           const double* d_mass);
nyxpm_status launch_pack(Ctx& c, Box& b, double* d_pos, double* d_vel);
nyxpm_status launch_wrap(Ctx& c, Box& b);
nyxpm_status launch_sort(Ctx& c, Box& b, bool defer_vel = false);
// the host-buffer step's split transfers (FP64 boxes)
nyxpm_status launch_unpack_pos(Ctx& c, Box& b, const double* d_pos, const double* d_mass);
nyxpm_status launch_unpack_gather_vel(Ctx& c, Box& b, const double* d_vel, bool sorted_since);
nyxpm_status launch_pack_pos_wrapped(Ctx& c, Box& b, double* d_pos);
nyxpm_status launch_pack_vel(Ctx& c, Box& b, double* d_vel);
nyxpm_status launch_deposit(Ctx& c, Box& b);
nyxpm_status launch_kick(Ctx& c, Box& b, double dt, double a_prev, double a_cur, int do_move,
                         int do_wrap);

nyxpm_status launch_make_rhs(Ctx& c, Box& b, double a);
// particle time-step limit into norms[3] (as ~bits of the minimum dt)
nyxpm_status launch_est_dt(Ctx& c, Box& b, double cfl, double a);
nyxpm_status mixed_est_dt(Ctx& c, Box& b, double cfl, double a);
double beta_scale(const Box& b);  // (h*h)/6 of level 0: rhs -> smoother units
nyxpm_status launch_zero_phi(Ctx& c, Box& b);
nyxpm_status mg_solve(Ctx& c, Box& b, nyxpm_solve_info* info);
nyxpm_status launch_grav_vector(Ctx& c, Box& b);
nyxpm_status launch_phi_to_natural(Ctx& c, Box& b, double* d_out);
nyxpm_status launch_phi_from_natural(Ctx& c, Box& b, const double* d_in);
// one V-cycle of b's hierarchy from a zero guess for the right-hand side beta
// (smoother units, natural layout), the correction into e (natural layout): the
// base level's correction solve of the multilevel composite V-cycle
nyxpm_status mg_vcycle_zero(Ctx& c, Box& b, const double* beta_nat, double* e_nat);

// mixed-precision form
nyxpm_status mixed_unpack(Ctx& c, Box& b, const double* d_pos, const double* d_vel,
                          const double* d_mass);
nyxpm_status mixed_pack(Ctx& c, Box& b, double* d_pos, double* d_vel);
nyxpm_status mixed_sort(Ctx& c, Box& b, bool defer_vel = false);
// the host-buffer step's split transfers (mixed boxes)
nyxpm_status mixed_unpack_pos(Ctx& c, Box& b, const double* d_pos, const double* d_mass);
nyxpm_status mixed_unpack_vel(Ctx& c, Box& b, const double* d_vel, bool sorted_since);
nyxpm_status mixed_pack_pos(Ctx& c, Box& b, double* d_pos);
nyxpm_status mixed_pack_vel(Ctx& c, Box& b, double* d_vel);
nyxpm_status mixed_deposit(Ctx& c, Box& b);
nyxpm_status mixed_kick(Ctx& c, Box& b, double dt, double a_prev, double a_cur, int do_move);
nyxpm_status mixed_solve(Ctx& c, Box& b, int zero_guess, nyxpm_solve_info* info);

nyxpm_status mixed_make_rhs(Ctx& c, Box& b, double a);
nyxpm_status mixed_grav32(Ctx& c, Box& b);  // FP32 gravity vector of the FP64 phi
nyxpm_status mixed_g32_from_g(Ctx& c, Box& b);  // FP32 gravity vector of the FP64 g
nyxpm_status mixed_rho_to_double(Ctx& c, Box& b);

// host-side helpers shared by the forms
nyxpm_status scan_counts(Ctx& c, Box& b);     // cell_count -> cell_start
nyxpm_status fix_segments(Ctx& c, Box& b);    // deterministic order inside each key segment
nyxpm_status sort_from_keys(Ctx& c, Box& b);  // key + cell_count -> perm (scan, scatter, fix)

}  // namespace nyxpm

struct nyxpm_ctx : public nyxpm::Ctx {};
struct nyxpm_box : public nyxpm::Box {};
