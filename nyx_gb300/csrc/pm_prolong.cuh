// FP32 trilinear prolongation of a split coarse level into the black cells of a
// split fine level, four fine rows per thread: the single-box kernel
// (k_prolong_f4_black) and the ensemble's (e_prolong4_black) share these helpers.
//
// The fine rows j = 2J, 2J + 1 of the planes k = 2K, 2K + 1 all draw on the coarse
// rows J - 1 .. J + 1 of the planes K - 1 .. K + 1, so one thread loads nine coarse
// row segments for four fine rows (one fine row per thread loads four for one).
// A thread covers four compact columns: eight fine cells of each row, of which
// the four black ones take the correction (post-smoothing follows, and its first,
// red, half sweep overwrites the red cells unread).  In the split layout those
// four are one float4 of the black array whichever colour the row starts with.
// Each black cell sums its eight weighted coarse values in the order of the
// one-row kernels (nearest coarse row and plane first, the x pair innermost), so
// the bits are theirs.
//
// LV is a level view with fields n, phi_r and phi_b (the red and black compact
// arrays, half = n / 2 values per row, rows x fastest, then y, then z).
#pragma once

namespace nyxpm {

// the trilinear weights of coarse neighbour tt + 2 a + 4 b (tt, a, b = 0: the
// nearer coarse cell along x, y, z): (3/4 or 1/4) per axis, as exact floats
// (one copy per translation unit that includes this header)
static __constant__ float kProlongQuadW[8] = {0.421875f, 0.140625f, 0.140625f, 0.046875f,
                                              0.140625f, 0.046875f, 0.046875f, 0.015625f};

// the six coarse values at I = ih0 - 1 .. ih0 + 4 of coarse row (J, K), c2 = the
// compact index of the even I = ih0
template <class LV>
__device__ __forceinline__ void prolong_row6(const LV& Cv, int J, int K, unsigned c2, float v[6])
{
    const unsigned chalf = (unsigned)Cv.n >> 1;
    const unsigned row = ((unsigned)J + (unsigned)Cv.n * (unsigned)K) * chalf;
    const bool even_red = ((J + K) & 1) == 0;   // colour of an even I
    const float* ev = even_red ? Cv.phi_r : Cv.phi_b;
    const float* od = even_red ? Cv.phi_b : Cv.phi_r;
    const float2 e01 = __ldg(reinterpret_cast<const float2*>(ev + row + c2));
    const float e2 = __ldg(ev + row + (c2 + 2 == chalf ? 0u : c2 + 2));
    const float2 o01 = __ldg(reinterpret_cast<const float2*>(od + row + c2));
    const float om = __ldg(od + row + (c2 == 0 ? chalf - 1 : c2 - 1));
    v[0] = om;
    v[1] = e01.x;
    v[2] = o01.x;
    v[3] = e01.y;
    v[4] = o01.y;
    v[5] = e2;
}

// the black corrections of fine rows (2J + dj, 2K + DK), dj = 0, 1, from the coarse
// rows v[kk][jj] = (J - 1 + jj, K - 1 + kk): Js = {J, dj ? J + 1 : J - 1}, Ks
// likewise.  A row's even cells are red iff dj + DK is even, and then its black
// cells are the odd ones, else the even ones.
template <int DK, class LV>
__device__ __forceinline__ void prolong_black_rows(const float (&v)[3][3][6], const LV& F, int J, int K,
                                                   unsigned t4)
{
    const unsigned half = (unsigned)F.n >> 1;
#pragma unroll
    for (int dj = 0; dj < 2; ++dj) {
        const bool odd_black = ((dj + DK) & 1) == 0;
        float s[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            float acc = 0.f;
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const float* w = v[b ? (DK ? 2 : 0) : 1][a ? (dj ? 2 : 0) : 1];
                    acc = fmaf(kProlongQuadW[0 + 2 * a + 4 * b], w[r + 1], acc);
                    acc = fmaf(kProlongQuadW[1 + 2 * a + 4 * b], odd_black ? w[r + 2] : w[r], acc);
                }
            s[r] = acc;
        }
        const unsigned j = 2u * J + dj, k = 2u * K + DK;
        const unsigned t = (j + (unsigned)F.n * k) * half + 4 * t4;
        float4* fb = reinterpret_cast<float4*>(F.phi_b) + (t >> 2);
        float4 p = *fb;
        p.x += s[0]; p.y += s[1]; p.z += s[2]; p.w += s[3];
        *fb = p;
    }
}

// The four fine rows of coarse row (J, K) for compact column group t4 of a split
// fine level over a split coarse level (fine n % 8 == 0).  The plane K + 1 is
// loaded only after the rows of plane 2K are written, which keeps the register
// count at five 256-thread CTAs per SM.
template <class LV>
__device__ __forceinline__ void prolong_black_quad(const LV& Cv, const LV& F, int J, int K, unsigned t4)
{
    const int nc = Cv.n;
    const int Jr[3] = {J == 0 ? nc - 1 : J - 1, J, J + 1 == nc ? 0 : J + 1};
    const int Km = K == 0 ? nc - 1 : K - 1, Kp = K + 1 == nc ? 0 : K + 1;
    const unsigned c2 = 2 * t4;
    float v[3][3][6];
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
        prolong_row6(Cv, Jr[jj], Km, c2, v[0][jj]);
        prolong_row6(Cv, Jr[jj], K, c2, v[1][jj]);
    }
    prolong_black_rows<0>(v, F, J, K, t4);
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) prolong_row6(Cv, Jr[jj], Kp, c2, v[2][jj]);
    prolong_black_rows<1>(v, F, J, K, t4);
}

}  // namespace nyxpm
