// FP32 restriction helpers shared by the single-box kernel (k_restrict_f4_red)
// and the ensemble's (e_restrict4_red).  LV is a level view with fields n,
// phi_r, phi_b, beta_r (the red and black compact arrays of a split level,
// half = n / 2 values per row, rows x fastest, then y, then z).
#pragma once

namespace nyxpm {

constexpr float kRestrictSixth = 1.0f / 6.0f;

// The red cells' residuals of one fine row segment (cells 4t .. 4t+3 of row (j, k)):
// r[u] for the red cell of the pair (4t + 2u, 4t + 2u + 1).  After pre-smoothing,
// which ends with a black half sweep, the black cells' residuals are round-off,
// so the restriction takes the red children only: the red values of this row
// (phi and beta at red[2t], red[2t+1]), three black values of this row around
// them and the black values of the four neighbour rows at the same x.  The
// neighbour sum is formed in the order of the all-children residual (x-, x+, y-,
// y+, z-, z+).
template <class LV>
__device__ __forceinline__ void fine_row_resid_red(const LV& F, int j, int k, unsigned t,
                                                   float r[2])
{
    const int n = F.n;
    const unsigned half = (unsigned)n >> 1;
    const int p = (j + k) & 1;                    // 0: red cells at even i
    auto row = [&](int jj, int kk) -> unsigned { return ((unsigned)jj + (unsigned)n * (unsigned)kk) * half; };
    const unsigned r0 = row(j, k), c2 = 2 * t;
    const float2 self = __ldg(reinterpret_cast<const float2*>(F.phi_r + r0 + c2));
    const float2 beta = __ldg(reinterpret_cast<const float2*>(F.beta_r + r0 + c2));
    const float2 bl = __ldg(reinterpret_cast<const float2*>(F.phi_b + r0 + c2));   // black 2t, 2t+1
    // the black value one beyond the pair: 2t-1 (p = 0) or 2t+2 (p = 1), periodic
    const float edge = p ? __ldg(F.phi_b + r0 + (c2 + 2 == half ? 0u : c2 + 2))
                         : __ldg(F.phi_b + r0 + (c2 == 0 ? half - 1 : c2 - 1));
    const float xm[2] = {p ? bl.x : edge, p ? bl.y : bl.x};
    const float xp[2] = {p ? bl.y : bl.x, p ? edge : bl.y};
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    const unsigned nr[4] = {row(jm, k), row(jp, k), row(j, km), row(j, kp)};
    float2 nb[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) nb[a] = __ldg(reinterpret_cast<const float2*>(F.phi_b + nr[a] + c2));
    const float sv[2] = {self.x, self.y}, bv[2] = {beta.x, beta.y};
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        float s = xm[u] + xp[u];
#pragma unroll
        for (int a = 0; a < 4; ++a) s += u ? nb[a].y : nb[a].x;
        r[u] = bv[u] - fmaf(s, kRestrictSixth, -sv[u]);
    }
}

}  // namespace nyxpm
