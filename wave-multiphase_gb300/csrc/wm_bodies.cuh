// wm_bodies.cuh -- per-cell and per-face bodies of the stage kernels, shared by the per-solve
// kernels (wm_stage.cu, wm_faces.cu) and the batched persistent kernel (wm_batch.cu). Each body
// handles one cell (i, j) or the faces it owns; callers do the index mapping and range checks.
#pragma once
#include "wm_kernels.cuh"

namespace wm {

__device__ __forceinline__ long long kf_of(const Fields &q, int i, int j)
{
    return (long long)i * q.pitch + j;
}
__device__ __forceinline__ long long kw_of(const Grid &g, int i, int j)
{
    return (long long)i * g.nyg + j;
}

// Warp-aggregated counter increment (one atomic per warp).
__device__ __forceinline__ void count_if(unsigned long long *ctr, bool pred)
{
    unsigned mask = __activemask();
    unsigned b = __ballot_sync(mask, pred);
    if (b && (threadIdx.x & 31) == (__ffs(mask) - 1)) atomicAdd(ctr, (unsigned long long)__popc(b));
}

// The cell entropy of cell_entropy (SC:308-314), binary64: p / rho^gamma, gamma = gamma(alpha),
// with rho clamped below at 1e-20 as the reference clamps it.
__device__ __forceinline__ double entropy64_r(double ge, double rho_e, double pp) { return pp / pow(rho_e, ge); }
__device__ __forceinline__ double entropy64(double ge, double ar1, double ar2, double pp)
{
    double rho_e = ar1 + ar2;
    if (rho_e < kTiny) rho_e = kTiny;
    return entropy64_r(ge, rho_e, pp);
}

// Bit equality of two binary64 values, on the integer pipe.
__device__ __forceinline__ bool same_bits(double a, double b)
{
    return __double_as_longlong(a) == __double_as_longlong(b);
}

// The mixture gamma and p_inf of a cell from its Gamma and Pi (mix_gamma_pinf's formula, with the
// face sweep's refined reciprocal for 1 / (Gamma (1 + Gamma))): the one evaluation behind every
// binary64 entropy -- both forms' preparation, the switch pre-checks and their diagnostic -- so the
// THINC switch is decided on the same values in every form.
__device__ __forceinline__ void entropy_gamma(double gb, double pb, double &g, double &pi)
{
    mix_from_pibig<double, true>(gb, pb, g, pi);
}

// prim_to_energy (SC:105-110) from the mixture's Gamma and Pi: the same expression.
__device__ __forceinline__ double energy_gp(double gb, double pb, double rho, double u, double v, double p)
{
    return gb * p + pb + 0.5 * rho * (u * u + v * v);
}

// A sensor value reduced to its side of the face sweep's threshold: 0 below it, 1 at or above it,
// NaN for NaN. The map is monotone, so it commutes with the reference's a<b?a:b minimum and maximum
// over the four cells of a face (NaN included), and (encoded < threshold) holds exactly when
// (value < threshold) does: the binary32 sweep makes the decisions of the binary64 values.
__device__ __forceinline__ float side_of(double v, double threshold)
{
    return v < threshold ? 0.0f : (isnan(v) ? __int_as_float(0x7fc00000) : 1.0f);
}

// ------------------------------------------------------------------------------------------------
// Binary32 pre-check of the THINC switch. The entropies reach the face sweep only through one
// comparison, cator2_val < 0.35 (SC:318-325, 1028-1032), so the sensor pass first makes it from
// binary32 entropies with an error bound, and falls back to the binary64 entropies (binary64 pow,
// as the reference) only where the bound does not settle it. The decision is the binary64 one in
// every case: the results are the same bits.
//
// entropy32: p / rho^gamma as p * 2^(-gamma log2 rho), from integer-pipe roundings of the binary64
// rho (already clamped), gamma and p. Relative error against p / rho^gamma of those binary64
// inputs, for |t| = |gamma log2 rho| <= 64 and gamma <= 64: the rounded rho moves log2 rho by
// 2^-23.47; log2f (1 ulp), the rounded gamma and the product move t by at most
// gamma 2^-23.47 + |t| 2^-22; exp2f (2 ulp), the rounded p and the final product add 2^-21.4; in
// all below 2^-21.4 + ln2 (gamma 2^-23.47 + |t| 2^-22) <= 1.6e-5. kEnt32Rel = 2^-14 is four
// times that (and covers the binary64 pow's few ulp). Outside those limits, or for operands that
// are not finite and normal (|p| in [2^-60, 2^60], so the result is normal too), it returns NaN:
// no pre-check with that cell. p = 0 gives the exact 0.
constexpr float kEnt32Rel = 6.1035156e-05f;  // 2^-14
__device__ __forceinline__ float entropy32(double ge, double rho_e, double pp)
{
    if ((__double_as_longlong(pp) << 1) == 0) return 0.0f;  // pp == 0, either sign
    const float r = to_f32(rho_e), gm = to_f32(ge), pf = to_f32(pp), ap = fabsf(pf);
    const float nan = __int_as_float(0x7fc00000);
    if (!(r >= 1.17549435e-38f && r <= 3.0e38f) || !(gm > 0.0f && gm <= 64.0f) ||
        !(ap >= 8.67361738e-19f && ap <= 1.15292150e18f))
        return nan;
    const float t = gm * log2f(r);
    if (!(fabsf(t) <= 64.0f)) return nan;
    return pf * exp2f(-t);
}

// The switch from five binary32 entropies: 0 (cator2 < 0.35) or 1 (>= 0.35) when the bound settles
// it, -1 when it does not (NaN entropies included). With a = aa and b = bb of cator2_val,
// cator2 < 0.35  <=>  f = 2ab - 0.35 (a^2 + b^2) + 0.65 eps < 0 (its denominator is positive).
// Each binary32 entropy is within kEnt32Rel of the binary64 one, so a is within
// da = (kEnt32Rel + 2^-20) Ma of the binary64 aa, Ma the sum of the magnitudes of aa's terms (2^-20
// covers the roundings of both evaluations of aa); b likewise. f is bounded over that box by
// interval arithmetic; a decision needs the whole interval, widened by 2^-19 of the magnitudes for
// the binary32 roundings of f, on one side of zero.
__device__ __forceinline__ int thinc_side_pre(float em2, float em1, float e0, float ep1, float ep2)
{
    const float k13 = 13.0f / 12.0f;
    const float a = 0.25f * fabsf(em2 - 4.0f * em1 + 3.0f * e0) + k13 * fabsf(e0 - 2.0f * em1 + em2);
    const float b = 0.25f * fabsf(3.0f * e0 - 4.0f * ep1 + ep2) + k13 * fabsf(e0 - 2.0f * ep1 + ep2);
    const float m2 = fabsf(em2), m1 = fabsf(em1), m0 = fabsf(e0), n1 = fabsf(ep1), n2 = fabsf(ep2);
    const float ma = 0.25f * (m2 + 4.0f * m1 + 3.0f * m0) + k13 * (m0 + 2.0f * m1 + m2);
    const float mb = 0.25f * (3.0f * m0 + 4.0f * n1 + n2) + k13 * (m0 + 2.0f * n1 + n2);
    const float rel = kEnt32Rel + 9.53674316e-07f;
    const float da = rel * ma, db = rel * mb;
    const float alo = fmaxf(a - da, 0.0f), ahi = a + da, blo = fmaxf(b - db, 0.0f), bhi = b + db;
    const float c = 0.65f * float(kYuxin);
    const float flo = 2.0f * alo * blo - 0.35f * (ahi * ahi + bhi * bhi) + c;
    const float fhi = 2.0f * ahi * bhi - 0.35f * (alo * alo + blo * blo) + c;
    const float m = 1.90734863e-06f * (2.0f * ahi * bhi + 0.35f * (ahi * ahi + bhi * bhi) + c);
    if (flo > m) return 1;
    if (fhi < -m) return 0;
    return -1;
}

// Second pre-check of the THINC switch, for the stencils the binary32 entropies leave: smooth flow
// with entropies far from 1 (air at 1 bar in SI units: about 8e4), where their relative bound
// swamps the second differences. The indicator depends on the entropies only through their ratios
// to the centre's: with r_k = e_k / e_0 = 1 + d_k, aa = |e_0| A and bb = |e_0| B, where
//   A = |d_-2 - 4 d_-1| / 4 + 13/12 |d_-2 - 2 d_-1|   (B likewise with d_2, d_1),
// so cator2 < 0.35  <=>  2AB - 0.35 (A^2 + B^2) + 0.65 eps / e_0^2 < 0. Each
//   d_k = expm1(L_k),  L_k = ln(e_k / e_0) = log1p(dp_k / p_0) - g_k log1p(dr_k / r_0) - dg_k ln r_0,
// an identity for e_k = p_k / r_k^g_k with the differences dp, dr (the clamped densities) and dg
// (the cells' binary64 mixture gammas) of the binary64 values, here taken from their binary32
// pairs x = hi + lo (split32, within 2^-48 |x|) as (hi_k - hi_0) + (lo_k - lo_0): within
// 2^-23 |dx| + 2^-46 (|x_k| + |x_0|) of the binary64 difference, and exactly 0 where the binary64
// values are equal -- a uniform region gives d = 0 exactly, as its binary64 entropies are equal. The
// rest is binary32, inside the ranges where the bound below holds (|dp / p_0|, |dr / r_0|,
// |L| <= 0.5). Error bound of d_k: the pair differences, the hi parts (the binary32 roundings of
// p_0, r_0, g_k), the reciprocals and the products put a quotient dp / p_0 within 2^-21.68 relative
// and 2^-44.6 absolute; log1p_pc and expm1_pc are within 2^-22.9 relative and logf within 1 ulp
// (CUDA's documented bound), and |x| <= 1.24 |log1p(x)| there; together |dL| <= 2^-19 (|log1p(xp)| +
// |g log1p(xr)| + |dg| (1 + |ln r_0|)) + 2^-43 (1 + g_k + (g_k + g_0) |ln r_0|) and
// |dd| <= 2^-22 |d| + 1.7 |dL|.
// A and B get those errors through their coefficients, 2^-21 of their magnitudes for their own
// roundings, and 2^-44 (6.4 + their magnitude) for the binary64 evaluation the decision must
// reproduce (pow within 2 ulp, the quotient, five roundings of aa). |e_0| comes from the binary32
// entropy (within kEnt32Rel). f is bounded over the box by interval arithmetic; a decision needs
// the interval clear of zero by 2^-18 of f's terms (binary32 roundings of f and the binary64
// quotient's). Returns 0 or 1 as the decision, -1 when undecided (NaN or out-of-range inputs
// included). No binary64 arithmetic.
// The stencil's pairs: at(k, PR_*) is the pair array's value at stencil cell k (0..4, centre 2) --
// read from prep's arrays as needed (PairsAt) or held in registers (SwitchPairs).
struct SwitchPairs {
    float v[6][5];
    __device__ __forceinline__ float operator()(int k, int w) const { return v[w][k]; }
};
struct PairsAt {
    float *const *pair;
    long long c0, stride;
    __device__ __forceinline__ float operator()(int k, int w) const { return pair[w][c0 + (k - 2) * stride]; }
};
template <typename At>
__device__ __forceinline__ int thinc_side_delta(const At &at, float e0)
{
    const float ae0 = fabsf(e0);
    if (!(ae0 > 0.0f) || !(ae0 <= 3.0e38f)) return -1;
    // |p_0|, r_0 >= 2^-60: a difference that is subnormal in binary32 then moves its quotient by
    // at most 2^-90, far inside the bound's binary64 floor below; with |dp / p_0|, |dr / r_0| <= 0.5
    // every pressure and density of the stencil lies in split32's domain (|x| >= 2^-74)
    const float p0 = at(2, PR_PH), r0 = at(2, PR_RH), g0 = at(2, PR_GH);
    const float pl0 = at(2, PR_PL), rl0 = at(2, PR_RL), gl0 = at(2, PR_GL);
    if (!(fabsf(p0) >= 8.67361738e-19f && fabsf(p0) <= 3.0e38f) || !(r0 >= 8.67361738e-19f && r0 <= 3.0e38f))
        return -1;
    const float lnr0 = logf(r0), w0 = 1.0f + fabsf(lnr0);
    const float ip0 = __frcp_rn(p0), ir0 = __frcp_rn(r0);  // correctly rounded reciprocals
    float d[5], D[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        if (k == 2) {
            d[k] = 0.0f;
            D[k] = 0.0f;
            continue;
        }
        const float dp = (at(k, PR_PH) - p0) + (at(k, PR_PL) - pl0);
        const float dr = (at(k, PR_RH) - r0) + (at(k, PR_RL) - rl0);
        const float gk = at(k, PR_GH);
        const float dgf = (gk - g0) + (at(k, PR_GL) - gl0);
        const float xp = dp * ip0, xr = dr * ir0;
        if (!(fabsf(xp) <= 0.5f) || !(fabsf(xr) <= 0.5f)) return -1;
        // gammas in [2^-60, 64]: inside split32's domain, and the bound's range
        if (!(gk >= 8.67361738e-19f && gk <= 64.0f) || !(g0 >= 8.67361738e-19f && g0 <= 64.0f) ||
            !(fabsf(dgf) <= 64.0f))
            return -1;
        const float lp = log1p_pc(xp), gl = gk * log1p_pc(xr), dl = dgf * lnr0;
        const float L = (lp - gl) - dl;
        if (!(fabsf(L) <= 0.5f)) return -1;
        const float dL = 1.9073486e-06f * (fabsf(lp) + fabsf(gl) + fabsf(dgf) * w0) +  // 2^-19
                         0x1p-43f * (1.0f + gk + (gk + g0) * fabsf(lnr0));
        d[k] = expm1_pc(L);
        D[k] = 2.3841858e-07f * fabsf(d[k]) + 1.7f * dL;  // 2^-22
    }
    const float k13 = 13.0f / 12.0f;
    const float A = 0.25f * fabsf(d[0] - 4.0f * d[1]) + k13 * fabsf(d[0] - 2.0f * d[1]);
    const float B = 0.25f * fabsf(d[4] - 4.0f * d[3]) + k13 * fabsf(d[4] - 2.0f * d[3]);
    const float MA = 0.25f * (fabsf(d[0]) + 4.0f * fabsf(d[1])) + k13 * (fabsf(d[0]) + 2.0f * fabsf(d[1]));
    const float MB = 0.25f * (fabsf(d[4]) + 4.0f * fabsf(d[3])) + k13 * (fabsf(d[4]) + 2.0f * fabsf(d[3]));
    const float wA = 0.25f * (D[0] + 4.0f * D[1]) + k13 * (D[0] + 2.0f * D[1]) + 4.7683716e-07f * MA +
                     5.6843419e-14f * (6.4f + MA);  // 2^-21, 2^-44
    const float wB = 0.25f * (D[4] + 4.0f * D[3]) + k13 * (D[4] + 2.0f * D[3]) + 4.7683716e-07f * MB +
                     5.6843419e-14f * (6.4f + MB);
    // 0.65 eps / e_0^2 with e_0 within kEnt32Rel (its square within 2^-12.9) and the roundings here
    float Ylo, Yhi;
    if (ae0 > 1.0e17f) {  // below 3e-37: bounded by [0, 1e-36]
        Ylo = 0.0f;
        Yhi = 1.0e-36f;
    } else {
        const float Y = (0.65f * float(kYuxin)) / (ae0 * ae0);  // +inf for |e_0| below ~5e-21
        Ylo = Y * (1.0f - 2.4414062e-04f);                       // 2^-12
        Yhi = Y * (1.0f + 2.4414062e-04f);
    }
    const float Alo = fmaxf(A - wA, 0.0f), Ahi = A + wA, Blo = fmaxf(B - wB, 0.0f), Bhi = B + wB;
    const float fmin = 2.0f * Alo * Blo - 0.35f * (Ahi * Ahi + Bhi * Bhi) + Ylo;
    const float fmax = 2.0f * Ahi * Bhi - 0.35f * (Alo * Alo + Blo * Blo) + Yhi;
    const float m = 3.8146973e-06f * (2.0f * Ahi * Bhi + 0.35f * (Ahi * Ahi + Bhi * Bhi) + Yhi);  // 2^-18
    if (!isfinite(A) || !isfinite(B) || !isfinite(wA) || !isfinite(wB)) return -1;
    if (fmin > m || (isinf(Ylo) && isfinite(Ahi) && isfinite(Bhi))) return 1;
    if (fmax < -m) return 0;
    return -1;
}

// The binary64 entropy of the cell at kf from its state: the mixture gamma of entropy_gamma and the
// clamped density, as the preparation pass evaluates them (the same bits).
__device__ __forceinline__ double cell_entropy64(const Eos &e, const Fields &q, long long c)
{
    double gb, pb, ge, pie;
    mix_gamma_pibig(e, q.f[F_AL][c], gb, pb);
    entropy_gamma(gb, pb, ge, pie);
    double rho_e = q.f[F_AR1][c] + q.f[F_AR2][c];
    if (flt(rho_e, kTiny)) rho_e = kTiny;
    return entropy64_r(ge, rho_e, q.f[F_P][c]);
}

// The THINC switch of the cell at kw (its state at kf) along one direction -- workspace stride sw,
// state stride sq. With the pre-checks, as side_of's code: the binary32 decision where it is
// settled, else the ratio pre-check's (thinc_side_delta), else cator2_val of the binary64
// entropies evaluated here from the cell state and prep's binary64 mixture gammas exactly as the
// binary64 form evaluates them. Without: cator2_val of the binary64 entropies prep kept for every
// cell -- the value itself in binary64 arrays (the reference's array), its code in binary32 ones.
template <typename PT>
__device__ __forceinline__ double thinc_side(const Eos &e, const Fields &q, const PrepT<PT> &p, long long kw,
                                             long long kf, long long sw, long long sq, bool prechecks)
{
    double v[5];
    if (prechecks) {
        float s[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) s[k] = p.ent32[kw + (k - 2) * sw];
        const int d = thinc_side_pre(s[0], s[1], s[2], s[3], s[4]);
        if (d >= 0) return float(d);
        // prep's pairs of the stencil's pressures, clamped densities and gammas
        const int d2 = thinc_side_delta(PairsAt{p.pair, kw, sw}, s[2]);
        if (d2 >= 0) return float(d2);
        // the binary64 entropies from the state, as prep evaluates them
#pragma unroll
        for (int k = 0; k < 5; ++k) v[k] = cell_entropy64(e, q, kf + (k - 2) * sq);
    } else {
#pragma unroll
        for (int k = 0; k < 5; ++k) v[k] = p.ent64[kw + (k - 2) * sw];
        if constexpr (sizeof(PT) == 8) return cator2_val(v[0], v[1], v[2], v[3], v[4]);
    }
    return side_of(cator2_val(v[0], v[1], v[2], v[3], v[4]), kThincThresh);
}

// What prep leaves for thinc_side: with the pre-checks the binary32 entropy and the cell's
// binary64 mixture gamma (the ratio pre-check's input, and with the cell state all that the binary64
// entropy of an undecided stencil needs); without, the binary64 entropy.
template <typename PT>
__device__ __forceinline__ void store_entropy_r(const PrepT<PT> &p, long long kw, double ge, double rho, double pp,
                                                bool prechecks)
{
    double rho_e = rho;
    if (flt(rho_e, kTiny)) rho_e = kTiny;
    if (prechecks) {
        p.ent32[kw] = entropy32(ge, rho_e, pp);
        split32(pp, p.pair[PR_PH][kw], p.pair[PR_PL][kw]);
        split32(rho_e, p.pair[PR_RH][kw], p.pair[PR_RL][kw]);
        split32(ge, p.pair[PR_GH][kw], p.pair[PR_GL][kw]);
    } else {
        p.ent64[kw] = entropy64_r(ge, rho_e, pp);
    }
}
template <typename PT>
__device__ __forceinline__ void store_entropy(const PrepT<PT> &p, long long kw, double ge, double ar1, double ar2,
                                              double pp, bool prechecks)
{
    store_entropy_r(p, kw, ge, ar1 + ar2, pp, prechecks);
}

// (x / d < c) as the reference evaluates it, x / d rounded, for d > 0 and c > 0: settled from the
// product c d when x is more than 2^-50 of it away (the quotient's and the product's roundings are
// 2^-53 each; the compares on the integer pipe), else by the division itself, out of line. NaN x
// takes the division (false).
static __device__ __noinline__ bool quotient_below_rare(double x, double d, double c) { return x / d < c; }
__device__ __forceinline__ bool floor_quotient_below(double x, double d, double c)
{
    const double cd = c * d;
    if (dlt(x, cd * (1.0 - 8.8817841970012523e-16))) return true;
    if (dlt(cd * (1.0 + 8.8817841970012523e-16), x)) return false;
    return quotient_below_rare(x, d, c);
}

// sound_speed_r's formula for the mixture (g, pi) the caller already holds: sqrt(max(g (p + pi) / rho,
// 1e-20)) with 1/rho supplied, the root refined from a binary32 seed (sqrt_nr).
__device__ __forceinline__ double sound_speed_gp(double g, double pi, double inv_rho, double p)
{
    double val = g * (p + pi) * inv_rho;
    if (flt(val, kTiny)) val = kTiny;
    return sqrt_nr(val);
}

// Entropy (SC:308-314) and the first-order HLLC cell state of fx_low_kernel (SC:1309-1327), both
// pure functions of one cell, computed once per cell instead of once per face that reads them.
__device__ __forceinline__ void prep_body(const Grid &g, const Eos &e, const Fields &q, const Prep &p, bool prechecks,
                                          int i, int j)
{
    long long kf = kf_of(q, i, j), kw = kw_of(g, i, j);
    double ar1 = q.f[F_AR1][kf], ar2 = q.f[F_AR2][kf], ru = q.f[F_RU][kf], rv = q.f[F_RV][kf];
    double pp = q.f[F_P][kf], al = q.f[F_AL][kf];

    double gb, pb, ge, pie;
    mix_gamma_pibig(e, al, gb, pb);
    entropy_gamma(gb, pb, ge, pie);
    store_entropy(p, kw, ge, ar1, ar2, pp, prechecks);

    double rho = ar1 + ar2;
    double ir = rcp_nr(rho);  // 1 / rho (the face sweep's refined reciprocal)
    double a = al;
    double gg = ge, pi = pie;
    if (!alpha_inside(al)) {  // a clamped fraction: its own mixture
        a = clamp01_pp(al);
        mix_gamma_pibig(e, a, gb, pb);
        entropy_gamma(gb, pb, gg, pi);
    }
    double pl = pp;
    if (wisnan(pl) || floor_quotient_below(pl + pi, gg - 1.0, kPpCtilde)) pl = kPpCtilde * (gg - 1.0) - pi;
    double u = ru * ir, v = rv * ir;
    p.lu[kw] = u;
    p.lv[kw] = v;
    p.lp[kw] = pl;
    p.la[kw] = a;
    p.lc[kw] = sound_speed_gp(gg, pi, ir, pl);  // the sound speed of the clamped cell's mixture
    p.lE[kw] = energy_gp(gb, pb, rho, u, v, pl);  // prim_to_energy with the mixture at hand
}

// The terms of the Ducros sensor of an interior cell (ducros_kernel, SC:875-916), binary64:
// sigma_x = (ax / (bx + 1e-30)) * (d2 / den), sigma_y likewise, d2 = div^2, den = d2 + curl^2 + 1e-30.
struct DucrosTerms {
    double ax, bx, ay, by, d2, den;
};
__device__ __forceinline__ DucrosTerms ducros_terms(const Fields &q, int i, int j)
{
    const double *U = q.f[F_U], *V = q.f[F_V], *P = q.f[F_P];
    long long kf = kf_of(q, i, j), Q = q.pitch;
    double der_ux = 0.5 * (-U[kf - Q] + U[kf + Q]);
    double der_vx = 0.5 * (-V[kf - Q] + V[kf + Q]);
    double der_uy = 0.5 * (-U[kf - 1] + U[kf + 1]);
    double der_vy = 0.5 * (-V[kf - 1] + V[kf + 1]);
    double div_u = der_ux + der_vy;
    double curl_u = der_vx - der_uy;
    DucrosTerms t;
    t.d2 = div_u * div_u;
    t.den = t.d2 + curl_u * curl_u + 1.0e-30;
    double p0 = P[kf];
    double pm2 = P[kf - 2 * Q], pm1 = P[kf - Q], pp1 = P[kf + Q], pp2 = P[kf + 2 * Q];
    t.ax = fabs(-pm2 + 16.0 * pm1 - 30.0 * p0 + 16.0 * pp1 - pp2);
    t.bx = fabs(pm2 + 16.0 * pm1 + 30.0 * p0 + 16.0 * pp1 + pp2);
    pm2 = P[kf - 2];
    pm1 = P[kf - 1];
    pp1 = P[kf + 1];
    pp2 = P[kf + 2];
    t.ay = fabs(-pm2 + 16.0 * pm1 - 30.0 * p0 + 16.0 * pp1 - pp2);
    t.by = fabs(pm2 + 16.0 * pm1 + 30.0 * p0 + 16.0 * pp1 + pp2);
    return t;
}

// The two Ducros sensors as the reference evaluates them.
__device__ __forceinline__ void ducros_xy(const Fields &q, int i, int j, double &sx, double &sy)
{
    const DucrosTerms t = ducros_terms(q, i, j);
    const double ducros = t.d2 / t.den;
    sx = (t.ax / (t.bx + 1.0e-30)) * ducros;
    sy = (t.ay / (t.by + 1.0e-30)) * ducros;
}

// The Ducros sensor's side of kSigmaSmooth, the only use the face sweep makes of it (the maximum
// over a face's four cells against 0.01). sigma = (a / (b + 1e-30)) (d2 / den) with every term
// non-negative, so sigma < 0.01 <=> a d2 < 0.01 (b + 1e-30) den up to the roundings of the two
// evaluations (three each from the shared b + 1e-30 and den on, 2^-53 apiece, no cancellation):
// where the products differ by more than 2^-45 the code is settled without the three divisions,
// elsewhere (and for NaN or overflow) sigma is evaluated as ducros_xy evaluates it.
__device__ __forceinline__ float sigma_side(double a, double b, double d2, double den)
{
    const double den_b = b + 1.0e-30;
    const double num = a * d2, thr = 0.01 * (den_b * den);
    if (num < thr * (1.0 - 2.8421709430404007e-14)) return 0.0f;
    if (num > thr * (1.0 + 2.8421709430404007e-14)) return 1.0f;
    return side_of((a / den_b) * (d2 / den), kSigmaSmooth);
}

// ------------------------------------------------------------------------------------------------
// Binary32 pre-check of the Ducros sensor's side of kSigmaSmooth. The face sweep uses sigma only
// through sigma < 0.01, so the sensor pass first makes that comparison from the binary32 roundings
// of the stencil's u, v and p (the binary32 form's cell copies, or to_f32 of the state) with an error
// bound, and evaluates the binary64 sigma (ducros_terms, sigma_side) only where the bound does not
// settle it. Where it decides, the decision is that of the binary64 evaluation: the same bits.
//
// Bound. The binary64 a = |-p_-2 + 16 p_-1 - 30 p_0 + 16 p_1 - p_2| (b with + signs) rounds at most 5
// times, each within 2^-53 of a partial sum bounded by M = |p_-2| + 16 |p_-1| + 30 |p_0| + 16 |p_1| +
// |p_2|; the binary32 one differs from the exact a of the binary64 pressures by the inputs' roundings
// (2^-24 of each, weighted: 2^-24 M) and its own (5 x 2^-24 M); with M computed in binary32 (within
// 2^-21.3 of M) both are inside E = 2^-20 M of the binary32 value -- also after E is added or
// subtracted in binary32. The velocity terms: div = 0.5 (u_1 - u_-1) + 0.5 (v_1 - v_-1) (curl alike)
// in binary64 within 2^-51.9 Mu, Mu = 0.5 (|u_1| + |u_-1| + |v_1| + |v_-1|), and in binary32 within
// 4 x 2^-24 Mu of the exact value, plus 2^-147 for inputs or results below binary32's normal range:
// both inside 2^-21 Mu + 2^-140. D = div^2 / (div^2 + curl^2 + 1e-30) rises with |div| and falls
// with |curl|, so its binary64 value (six roundings: within 2^-50.4) lies between D at the interval
// ends; evaluated in binary32 those are within 2^-21.6 relative and 2^-49 absolute (a square below
// the normal range moves D by at most 2^-150 / 1e-30), covered by the factors 1 -+ 2^-20 and 2^-48.
// sigma = (a / (b + 1e-30)) D in binary64 is within 2^-50 of its exact value, so sigma < 0.01 holds
// when a_hi D_hi < 0.01 (1 - 2^-18) b_lo, and sigma >= 0.01 when a_lo D_lo > 0.01 (1 + 2^-18)
// (b_hi + 1e-30): the margins cover the products' binary32 roundings and 0.01f against 0.01. No
// decision for M outside [2^-90, 2^100] (relative bounds; no overflow), Mu or Mc above 2^60 (squares
// in range), b_lo below 2^-100 (the products stay normal where it matters), or NaN anywhere.
__device__ __forceinline__ float f32_of(float x) { return x; }
__device__ __forceinline__ float f32_of(double x) { return to_f32(x); }

// The pressure terms of one direction: bounds on the binary64 a and b; false where they do not hold.
__device__ __forceinline__ bool ducros_ab(float pm2, float pm1, float p0, float pp1, float pp2, float &alo,
                                          float &ahi, float &blo, float &bhi)
{
    const float a = fabsf(-pm2 + 16.0f * pm1 - 30.0f * p0 + 16.0f * pp1 - pp2);
    const float b = fabsf(pm2 + 16.0f * pm1 + 30.0f * p0 + 16.0f * pp1 + pp2);
    const float M = fabsf(pm2) + 16.0f * fabsf(pm1) + 30.0f * fabsf(p0) + 16.0f * fabsf(pp1) + fabsf(pp2);
    const float E = 0x1p-20f * M;
    alo = fmaxf(a - E, 0.0f);
    ahi = a + E;
    blo = b - E;
    bhi = b + E;
    return M >= 0x1p-90f && M <= 0x1p100f;
}

__device__ __forceinline__ int ducros_decide(bool ok, float alo, float ahi, float blo, float bhi, float Dlo, float Dhi)
{
    if (!ok) return -1;
    if (blo >= 0x1p-100f && ahi * Dhi < 0.009999962f * blo) return 0;  // 0.01 (1 - 2^-18)
    if (alo * Dlo > 0.010000038f * (bhi + 1.0e-30f)) return 1;           // 0.01 (1 + 2^-18)
    return -1;
}

// Both directions' pre-check codes (0, 1, or -1 undecided) of the cell at k, from arrays of binary64
// (converted here) or binary32 roundings, with strides sx, sy between x and y neighbours.
template <typename T>
__device__ __forceinline__ void ducros_pre(const T *U, const T *V, const T *P, long long k, long long sx,
                                           long long sy, int &dx, int &dy)
{
    const float uxm = f32_of(U[k - sx]), uxp = f32_of(U[k + sx]), uym = f32_of(U[k - sy]), uyp = f32_of(U[k + sy]);
    const float vxm = f32_of(V[k - sx]), vxp = f32_of(V[k + sx]), vym = f32_of(V[k - sy]), vyp = f32_of(V[k + sy]);
    const float div = 0.5f * (-uxm + uxp) + 0.5f * (-vym + vyp);
    const float curl = 0.5f * (-vxm + vxp) - 0.5f * (-uym + uyp);
    const float Mu = 0.5f * (fabsf(uxm) + fabsf(uxp) + fabsf(vym) + fabsf(vyp));
    const float Mc = 0.5f * (fabsf(vxm) + fabsf(vxp) + fabsf(uym) + fabsf(uyp));
    const float Ed = fmaf(0x1p-21f, Mu, 0x1p-140f), Ec = fmaf(0x1p-21f, Mc, 0x1p-140f);
    const float dlo = fmaxf(fabsf(div) - Ed, 0.0f), dhi = fabsf(div) + Ed;
    const float clo = fmaxf(fabsf(curl) - Ec, 0.0f), chi = fabsf(curl) + Ec;
    const float dlo2 = dlo * dlo, dhi2 = dhi * dhi;
    const float Dlo = fmaxf(fmaf(dlo2 / (dlo2 + chi * chi + 1.0e-30f), 1.0f - 0x1p-20f, -0x1p-48f), 0.0f);
    const float Dhi = fmaf(dhi2 / (dhi2 + clo * clo + 1.0e-30f), 1.0f + 0x1p-20f, 0x1p-48f);
    const bool okv = Mu <= 0x1p60f && Mc <= 0x1p60f;
    const float p0 = f32_of(P[k]);
    float alo, ahi, blo, bhi;
    bool ok = okv && ducros_ab(f32_of(P[k - 2 * sx]), f32_of(P[k - sx]), p0, f32_of(P[k + sx]), f32_of(P[k + 2 * sx]),
                               alo, ahi, blo, bhi);
    dx = ducros_decide(ok, alo, ahi, blo, bhi, Dlo, Dhi);
    ok = okv && ducros_ab(f32_of(P[k - 2 * sy]), f32_of(P[k - sy]), p0, f32_of(P[k + sy]), f32_of(P[k + 2 * sy]),
                          alo, ahi, blo, bhi);
    dy = ducros_decide(ok, alo, ahi, blo, bhi, Dlo, Dhi);
}

// Both Ducros sensors' codes of an interior cell: the binary32 pre-check's decisions from the
// arrays U, V, P (k, sx, sy as ducros_pre), the binary64 sigma_side where it leaves one open.
template <typename T>
__device__ __forceinline__ void ducros_sides_pre(const Fields &q, int i, int j, const T *U, const T *V, const T *P,
                                                 long long k, long long sx, long long sy, float &cx, float &cy)
{
    int dx, dy;
    ducros_pre(U, V, P, k, sx, sy, dx, dy);
    if (dx >= 0 && dy >= 0) {
        cx = float(dx);
        cy = float(dy);
        return;
    }
    const DucrosTerms t = ducros_terms(q, i, j);
    cx = dx >= 0 ? float(dx) : sigma_side(t.ax, t.bx, t.d2, t.den);
    cy = dy >= 0 ? float(dy) : sigma_side(t.ay, t.by, t.d2, t.den);
}

// The THINC switch per cell and direction (cator2_val < 0.35, SC:318-325, 1028-1032) and the
// Ducros x pressure sensor (ducros_kernel, SC:875-916): as side_of's codes with the pre-checks,
// the reference's values without.
__device__ __forceinline__ void sensor_body(const Grid &g, const Eos &e, const Fields &q, const Prep &p, int sc,
                                            bool prechecks, int i, int j)
{
    long long kw = kw_of(g, i, j), kf = kf_of(q, i, j);
    const long long W = g.nyg;
    if (i >= 2 && i < g.nxg - 2) p.cx[kw] = thinc_side(e, q, p, kw, kf, W, q.pitch, prechecks);
    if (j >= 2 && j < g.nyg - 2) p.cy[kw] = thinc_side(e, q, p, kw, kf, 1, 1, prechecks);
    if (!sc) return;
    if (i < 2 || i >= g.nxg - 2 || j < 2 || j >= g.nyg - 2) {
        p.sx[kw] = 1.0;
        p.sy[kw] = 1.0;
        return;
    }
    if (prechecks) {
        float cx, cy;
        ducros_sides_pre(q, i, j, q.f[F_U], q.f[F_V], q.f[F_P], kf, q.pitch, 1, cx, cy);
        p.sx[kw] = cx;
        p.sy[kw] = cy;
    } else {
        ducros_xy(q, i, j, p.sx[kw], p.sy[kw]);
    }
}

// Face limiter factors of pass p (pp_blend_x/y_flux_kernel, SC:1479-1548): the x face between
// cells (i, j) and (i+1, j) takes min(1, theta(i, j), theta(i+1, j)) over its interior neighbours,
// in that order; the y face between (i, j) and (i, j+1) likewise. Shared by blend_body, which
// writes the blended fluxes, and CellFaces, which rebuilds them in registers.
// The factors are stored in the flux type: rounding to binary32 is monotone, so the minimum of the
// rounded factors is the rounded minimum and the blends see the same values either way.
template <typename FT>
__device__ __forceinline__ FT face_theta_x(const Grid &g, const FT *theta, long long kw, int i)
{
    FT th = FT(1);
    if (i >= g.g) th = wmin(th, theta[kw]);
    if (i + 1 < g.g + g.nx) th = wmin(th, theta[kw + g.nyg]);
    return th;
}
template <typename FT>
__device__ __forceinline__ FT face_theta_y(const Grid &g, const FT *theta, long long kw, int j)
{
    FT th = FT(1);
    if (j >= g.g) th = wmin(th, theta[kw]);
    if (j + 1 < g.g + g.ny) th = wmin(th, theta[kw + 1]);
    return th;
}

// The first-order sides of a face (fx_low_kernel's states, SC:1309-1327): cells 0 and 1's partial
// densities and the preparation pass's first-order cell states (normal and tangential velocity,
// floored pressure, clamped alpha, sound speed, energy). One builder for the sweep and for the
// first-order values formed on demand, so both give the same bits.
template <typename T>
__device__ __forceinline__ void first_order_side(T ar1, T ar2, T un, T ut, T p, T a, T c, T E, Side<T> &S)
{
    S.ar1 = ar1; S.ar2 = ar2; S.rho = ar1 + ar2;
    S.un = un; S.ut = ut; S.p = p; S.a = a; S.c = c; S.E = E;
}

// The seven first-order values of the face between the cell at (kw0 in the padded grid, kf0 in the
// state) and its neighbour along DIR, formed from the face's LowSrc as the sweep forms them.
template <int DIR>
__device__ __forceinline__ void low_flux_on_demand(const LowSrc &s, long long kw0, long long kf0, double out[7])
{
    const long long sw = DIR == 0 ? s.nyg : 1, sf = DIR == 0 ? s.pitch : 1;
    const double *un = DIR == 0 ? s.lu : s.lv, *ut = DIR == 0 ? s.lv : s.lu;
    Side<double> L, R;
    first_order_side(s.ar1[kf0], s.ar2[kf0], un[kw0], ut[kw0], s.lp[kw0], s.la[kw0], s.lc[kw0], s.lE[kw0], L);
    const long long k1 = kw0 + sw, f1 = kf0 + sf;
    first_order_side(s.ar1[f1], s.ar2[f1], un[k1], ut[k1], s.lp[k1], s.la[k1], s.lc[k1], s.lE[k1], R);
    double f[6], us;
    hllc<DIR>(L, R, f, us);
#pragma unroll
    for (int c = 0; c < 6; ++c) out[c] = f[c];
    out[6] = us;
}

// The four faces of interior cell (i, j) with NP limiter passes deferred: the flux a face holds
// after passes 0..NP-1 is rebuilt from its high- and first-order values and the passes' cell
// factors by the same face_blend chain blend_body applies in place, so the values are identical
// bit for bit -- and the three blend sweeps over 28 face arrays are not needed. NP = 0 reads the
// (already blended, or not yet limited) high-order arrays as they are.
template <typename FT, int NP>
struct CellFaces {
    long long kw, kx, ky;
    FT txp[NP > 0 ? NP : 1], txm[NP > 0 ? NP : 1], typ[NP > 0 ? NP : 1], tym[NP > 0 ? NP : 1];

    __device__ __forceinline__ CellFaces(const Grid &g, FT *const theta[3], int i, int j)
    {
        kw = kw_of(g, i, j);
        kx = kw - g.nyg;
        ky = kw - 1;
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            txp[p] = face_theta_x(g, theta[p], kw, i);
            txm[p] = face_theta_x(g, theta[p], kx, i - 1);
            typ[p] = face_theta_y(g, theta[p], kw, j);
            tym[p] = face_theta_y(g, theta[p], ky, j - 1);
        }
    }
    // Binary64: a pass at theta = 1 on a face whose first-order values are all finite leaves the
    // value as it is (face_blend's rule), so the first-order value is read only for the other
    // passes. Binary32: every pass blends (face_blend's formula).
    __device__ __forceinline__ FT chain(const FT *hi, const FT *lo, const unsigned char *fin, long long k,
                                        const FT *t) const
    {
        FT v = hi[k];
        bool lofin = false;
        if (NP > 0 && sizeof(FT) == 8) lofin = fin[k] != 0;
#pragma unroll
        for (int p = 0; p < NP; ++p)
            if (!keeps_high(t[p], lofin)) v = face_blend(lo[k], v, t[p]);
        return v;
    }
    __device__ __forceinline__ FT xp(const Face<FT> &h, const Face<FT> &l, int c) const { return chain(h.f[c], l.f[c], l.fin, kw, txp); }
    __device__ __forceinline__ FT xm(const Face<FT> &h, const Face<FT> &l, int c) const { return chain(h.f[c], l.f[c], l.fin, kx, txm); }
    __device__ __forceinline__ FT yp(const Face<FT> &h, const Face<FT> &l, int c) const { return chain(h.f[c], l.f[c], l.fin, kw, typ); }
    __device__ __forceinline__ FT ym(const Face<FT> &h, const Face<FT> &l, int c) const { return chain(h.f[c], l.f[c], l.fin, ky, tym); }
};

// Binary32 pre-check of a limiter pass (precision form). The pass's factor is exactly 1 when the
// binary64 low- and high-order states l = Q - dt R_L, h = Q - dt R_H are finite and h clears the
// pass's bound (theta_cons_stage, SC:268-292; for pass 2, the division-free test of theta_ctilde).
// The same states formed in binary32 from the stage-start binary32 copies of Q differ from them by
// at most 3 * 2^-24 (|Q| + |dt R|) each (the rounding of Q and dt to binary32 and of the
// multiply-add, 1.8e-7 of those magnitudes); every test below demands a margin of 3e-7 of them,
// and for pass 2 a first-order bound of how those input errors and the binary32 evaluation move
// the test's value, doubled. When this returns true the binary64 bound solve would return 1, so
// it is skipped; otherwise the caller runs it. The results are the same bits either way.
template <int STAGE>
__device__ __forceinline__ bool theta_one_core(const Eos &e, const float *hx, const float *dx, bool lfin)
{
    if (!lfin) return false;
    if (STAGE == 0) {
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 2; ++k) ok = ok && isfinite(hx[k]) && hx[k] >= float(kPpRho) * 1.000001f + dx[k];
        return ok;
    } else if (STAGE == 1) {
        const float lo = float(kPpAlpha) * 1.000001f + dx[5];
        return isfinite(hx[5]) && hx[5] >= lo && 1.0f - hx[5] >= lo;
    } else {
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 6; ++k) ok = ok && isfinite(hx[k]);
        if (!ok) return false;
        // ctilde_surely_above in binary32: V = 2 rho (1+G)(E - floor) - (1+G)(mx^2+my^2) - 2 rho Pi
        float a1 = hx[5];
        if (a1 < float(kPpAlpha)) a1 = float(kPpAlpha);
        if (a1 > 1.0f - float(kPpAlpha)) a1 = 1.0f - float(kPpAlpha);
        const float m1 = fmaxf(hx[0], float(kPpRho)), m2 = fmaxf(hx[1], float(kPpRho));
        const float rho = m1 + m2, a2 = 1.0f - a1;
        const float gb = a1 * e.r1f + a2 * e.r2f, pb = a1 * e.k1f + a2 * e.k2f, gp1 = 1.0f + gb;
        const float Ef = hx[4] - float(kPpCtilde);
        const float mom = hx[2] * hx[2] + hx[3] * hx[3];
        const float t1 = 2.0f * rho * gp1 * Ef, t2 = gp1 * mom, t3 = 2.0f * rho * pb;
        const float V = t1 - t2 - t3;
        const float T = fabsf(t1) + t2 + fabsf(t3);
        // first-order movement of V under the input errors (upper bounds of the magnitudes)
        const float drho = dx[0] + dx[1];
        const float rho_u = rho + drho, E_u = fabsf(Ef) + dx[4];
        const float mx_u = fabsf(hx[2]) + dx[2], my_u = fabsf(hx[3]) + dx[3];
        const float dV = (2.0f * gp1 * E_u + 2.0f * fabsf(pb)) * drho + 2.0f * rho_u * gp1 * dx[4] +
                         2.0f * gp1 * (mx_u * dx[2] + my_u * dx[3]) +
                         (fabsf(e.r1f - e.r2f) * (2.0f * rho_u * E_u + mx_u * mx_u + my_u * my_u) +
                          2.0f * rho_u * fabsf(e.k1f - e.k2f)) * dx[5];
        return isfinite(V) && isfinite(T) && isfinite(dV) && V > 2.0f * dV + 1.0e-6f * T;
    }
}

// Precision form: the binary32 states from the stage-start binary32 copies and the binary32
// residuals the binary64 solve would widen (margin 3e-7 of |Q| + |dt R|).
template <int STAGE>
__device__ __forceinline__ bool theta_one_f32(const Eos &e, const Cells32 &c, long long kw, const float *rh,
                                              const float *rl, float dtf)
{
    constexpr float kRel = 3.0e-7f;
    constexpr int C0 = STAGE == 1 ? 5 : 0, C1 = STAGE == 0 ? 2 : 6;
    const float *src[6] = {c.ar1, c.ar2, c.ru, c.rv, c.E, c.al};
    float hx[6], dx[6];
    bool lfin = true;
#pragma unroll
    for (int k = C0; k < C1; ++k) {
        const float qv = src[k][kw];
        const float dh = dtf * rh[k];
        hx[k] = qv - dh;
        dx[k] = kRel * (fabsf(qv) + fabsf(dh));
        if (STAGE != 2 || (k >= 2 && k <= 4)) lfin = lfin && isfinite(qv - dtf * rl[k]);
    }
    return theta_one_core<STAGE>(e, hx, dx, lfin);
}

__device__ __forceinline__ bool finite64(double x)
{
    return (__double_as_longlong(x) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
}

// Plain form (blends in place): the binary32 states from binary32 roundings of the binary64 state
// and face fluxes (integer-pipe conversions). Each face value is rounded by 2^-24 of itself, so the
// residual's error is bounded by its magnitude A = (|F+| + |F-|)/dx + (|G+| + |G-|)/dy (+ the
// alpha term's), and the state's by about 6 * 2^-24 (|Q| + dt A); the margin is 1e-6 of that.
// The low-order state is finite when its inputs are: the state and the first-order values of the
// four faces (the sweep's per-face bytes).
template <int STAGE>
__device__ __forceinline__ bool theta_one_f64in(const Grid &g, const Eos &e, const Fields &q, long long kf,
                                                long long kw, const Face<double> &fh, const Face<double> &gh,
                                                const Face<double> &fl, const Face<double> &gl, double dt)
{
    constexpr int C0 = STAGE == 1 ? 5 : 0, C1 = STAGE == 0 ? 2 : 6;
    const long long kx = kw - g.nyg, ky = kw - 1;
    const float dtf = to_f32(dt), idx = g.inv_dxf, idy = g.inv_dyf;
    float hx[6], dx[6];
    // every first-order value of the four faces finite (the sweep's bytes; stricter than the
    // components the pass uses, which only sends more cells to the binary64 solve)
    bool lfin = fl.fin[kw] && fl.fin[kx] && gl.fin[kw] && gl.fin[ky];
#pragma unroll
    for (int k = C0; k < C1; ++k) {
        const float xp = to_f32(fh.f[k][kw]), xm = to_f32(fh.f[k][kx]);
        const float yp = to_f32(gh.f[k][kw]), ym = to_f32(gh.f[k][ky]);
        float rh = div_sum(xp - xm, idx, yp - ym, idy);
        float A = (fabsf(xp) + fabsf(xm)) * idx + (fabsf(yp) + fabsf(ym)) * idy;
        const double qd = q.f[k][kf];
        bool fin = finite64(qd);
        if (k == 5) {
            const float a = to_f32(q.f[F_ALP][kf]);
            const float sxp = to_f32(fh.f[6][kw]), sxm = to_f32(fh.f[6][kx]);
            const float syp = to_f32(gh.f[6][kw]), sym = to_f32(gh.f[6][ky]);
            rh = rh - src_term(a, sxp - sxm, idx) - src_term(a, syp - sym, idy);
            A += fabsf(a) * ((fabsf(sxp) + fabsf(sxm)) * idx + (fabsf(syp) + fabsf(sym)) * idy);
            fin = fin && finite64(q.f[F_ALP][kf]);
        }
        const float qv = to_f32(qd);
        hx[k] = qv - dtf * rh;
        dx[k] = 1.0e-6f * (fabsf(qv) + dtf * A);
        lfin = lfin && fin && isfinite(A) && isfinite(dx[k]);
    }
    return theta_one_core<STAGE>(e, hx, dx, lfin);
}

// pp_cell_theta_kernel (SC:1397-1476): residuals of the current (partly blended) high-order and of
// the first-order fluxes, bound solve of this pass. Pass 0 bounds the partial densities, pass 1
// alpha and 1 - alpha, pass 2 rho c~^2 (theta_cons_stage, SC:268-292); each pass forms only the
// residual components its bound uses. NP: limiter passes whose blends are deferred (0 when the
// high-order arrays already hold the blended fluxes, STAGE when they are rebuilt in registers).
// The binary32 pre-checks above decide most cells without the binary64 solve (precision form:
// theta_one_f32; plain form with blends in place: theta_one_f64in); VERIFY runs the binary64 solve
// as well and counts (verify[0]) cells the pre-check decided and (verify[1]) cells where the solve
// disagreed with it -- a diagnostic of the pre-check's margins.
// The binary64 bound solve of one cell (after any binary32 pre-check), binary32 pre-check of the
// precision form included. OD: the first-order values may be formed on demand (Face::src.on);
// instantiations that never do (the batched kernel) are compiled without that code.
template <int STAGE, typename FT, int NP, int VERIFY, bool OD = false>
__device__ __forceinline__ double theta_solve_inline(const Grid &g, const Eos &e, const Fields &q, const Cells32 &c32,
                                                     const Face<FT> &fh, const Face<FT> &gh,
                                                     const Face<FT> &fl, const Face<FT> &gl, double dt,
                                                     FT *const theta[3], int i, int j,
                                                     unsigned long long *verify, bool prechecks, bool one = false)
{
    const CellFaces<FT, NP> cf(g, theta, i, j);
    const long long kf = kf_of(q, i, j), kw = cf.kw, kx = cf.kx, ky = cf.ky;
    const FT idx = cst<FT>(g.inv_dx, g.inv_dxf), idy = cst<FT>(g.inv_dy, g.inv_dyf);
    constexpr int C0 = STAGE == 1 ? 5 : 0, C1 = STAGE == 0 ? 2 : 6;
    FT rh[6], rl[6];
    // the first-order values of the four faces: formed here when the sweep left them unwritten
    // (binary64 fused stage), else read
    FT lxp[7], lxm[7], lyp[7], lym[7];
    bool formed = false;
    if constexpr (OD && sizeof(FT) == 8 && NP == 0) {
        if (fl.src.on) {
            low_flux_on_demand<0>(fl.src, kw, kf, lxp);
            low_flux_on_demand<0>(fl.src, kx, kf - q.pitch, lxm);
            low_flux_on_demand<1>(gl.src, kw, kf, lyp);
            low_flux_on_demand<1>(gl.src, ky, kf - 1, lym);
            formed = true;
        }
    }
#pragma unroll
    for (int c = C0; c < C1; ++c) {
        rh[c] = div_sum(cf.xp(fh, fl, c) - cf.xm(fh, fl, c), idx, cf.yp(gh, gl, c) - cf.ym(gh, gl, c), idy);
        if (formed)
            rl[c] = div_sum(lxp[c] - lxm[c], idx, lyp[c] - lym[c], idy);
        else
            rl[c] = div_sum(fl.f[c][kw] - fl.f[c][kx], idx, gl.f[c][kw] - gl.f[c][ky], idy);
        if (c == 5) {
            FT a;
            if constexpr (sizeof(FT) == 4) a = to_f32(q.f[F_ALP][kf]);
            else a = q.f[F_ALP][kf];
            rh[c] = rh[c] - src_term(a, cf.xp(fh, fl, 6) - cf.xm(fh, fl, 6), idx) -
                    src_term(a, cf.yp(gh, gl, 6) - cf.ym(gh, gl, 6), idy);
            if (formed)
                rl[c] = rl[c] - src_term(a, lxp[6] - lxm[6], idx) - src_term(a, lyp[6] - lym[6], idy);
            else
                rl[c] = rl[c] - src_term(a, fl.f[6][kw] - fl.f[6][kx], idx) -
                        src_term(a, gl.f[6][kw] - gl.f[6][ky], idy);
        }
    }
    if constexpr (sizeof(FT) == 4) {
        one = theta_one_f32<STAGE>(e, c32, kw, rh, rl, to_f32(dt));
        if (!VERIFY && one && prechecks) return 1.0;
    }
    double l[6], h[6];
#pragma unroll
    for (int c = C0; c < C1; ++c) {
        double qc = q.f[c][kf];
        double rlc, rhc;
        if constexpr (sizeof(FT) == 4) {
            rlc = to_f64(rl[c]);
            rhc = to_f64(rh[c]);
        } else {
            rlc = rl[c];
            rhc = rh[c];
        }
        l[c] = __fma_rn(-dt, rlc, qc);
        h[c] = __fma_rn(-dt, rhc, qc);
    }
    double th;
    if (STAGE == 2) {
        th = theta_ctilde(e, l, h);
    } else {
        th = theta_cons_stage(e, l, h, STAGE);
    }
    if (VERIFY && verify) {
        count_if(&verify[0], one);
        count_if(&verify[1], one && th != 1.0);
    }
    return th;
}

template <int STAGE, int VERIFY, bool OD>
__device__ __noinline__ double theta_solve(const Grid &g, const Eos &e, const Fields &q, const Face<double> fh,
                                           const Face<double> gh, const Face<double> fl, const Face<double> gl,
                                           double dt, int i, int j, unsigned long long *verify, bool one)
{
    double *const none[3] = {nullptr, nullptr, nullptr};
    return theta_solve_inline<STAGE, double, 0, VERIFY, OD>(g, e, q, Cells32{}, fh, gh, fl, gl, dt, none, i, j,
                                                             verify, false, one);
}

template <int STAGE, typename FT, int NP = 0, int VERIFY = 0, bool OD = false>
__device__ __forceinline__ double theta_body(const Grid &g, const Eos &e, const Fields &q, const Cells32 &c32,
                                             const Face<FT> &fh, const Face<FT> &gh,
                                             const Face<FT> &fl, const Face<FT> &gl, double dt,
                                             FT *const theta[3], int i, int j,
                                             unsigned long long *verify = nullptr, bool prechecks = true)
{
    bool one = false;
    if constexpr (sizeof(FT) == 8 && NP == 0) {  // plain form, blends in place
        const long long kf = kf_of(q, i, j), kw = kw_of(g, i, j);
        one = theta_one_f64in<STAGE>(g, e, q, kf, kw, fh, gh, fl, gl, dt);
        if (!VERIFY && one && prechecks) return 1.0;
        // the rare cells the pre-check leaves: out of line, so its registers do not hold down the
        // occupancy of the pass
        return theta_solve<STAGE, VERIFY, OD>(g, e, q, fh, gh, fl, gl, dt, i, j, verify, one);
    } else {
        return theta_solve_inline<STAGE, FT, NP, VERIFY>(g, e, q, c32, fh, gh, fl, gl, dt, theta, i, j, verify,
                                                         prechecks);
    }
}

// pp_blend_x_flux_kernel + pp_blend_y_flux_kernel (SC:1479-1548) in one launch: the thread at
// (i, j) blends x-face (i, j) and y-face (i, j) when they exist. OD as for theta_solve_inline.
template <typename FT, bool OD = false>
__device__ __forceinline__ void blend_body(const Grid &g, const Face<FT> &fh, const Face<FT> &gh,
                                           const Face<FT> &fl, const Face<FT> &gl,
                                           const FT *theta, int i, int j)
{
    long long kw = kw_of(g, i, j);
    // Binary64: a face at theta = 1 whose low-order values are all finite keeps its high-order
    // values (face_blend's value there): only its theta and its finiteness byte are read, nothing
    // is written. Binary32: the formula on every face.
    if (j >= g.g) {  // x face between (i, j) and (i+1, j)
        const FT t = face_theta_x(g, theta, kw, i);
        if (!(sizeof(FT) == 8 && keeps_high(t, fl.fin[kw] != 0))) {
            if constexpr (OD && sizeof(FT) == 8) {
                if (fl.src.on) {  // the first-order values formed here (binary64 fused stage)
                    double low[7];
                    low_flux_on_demand<0>(fl.src, kw, (long long)i * fl.src.pitch + j, low);
#pragma unroll
                    for (int c = 0; c < 7; ++c) fh.f[c][kw] = face_blend(low[c], fh.f[c][kw], t);
                    goto y_face;
                }
            }
#pragma unroll
            for (int c = 0; c < 7; ++c) fh.f[c][kw] = face_blend(fl.f[c][kw], fh.f[c][kw], t);
        }
    }
y_face:
    if (i >= g.g) {  // y face between (i, j) and (i, j+1)
        const FT t = face_theta_y(g, theta, kw, j);
        if (!(sizeof(FT) == 8 && keeps_high(t, gl.fin[kw] != 0))) {
            if constexpr (OD && sizeof(FT) == 8) {
                if (gl.src.on) {
                    double low[7];
                    low_flux_on_demand<1>(gl.src, kw, (long long)i * gl.src.pitch + j, low);
#pragma unroll
                    for (int c = 0; c < 7; ++c) gh.f[c][kw] = face_blend(low[c], gh.f[c][kw], t);
                    return;
                }
            }
#pragma unroll
            for (int c = 0; c < 7; ++c) gh.f[c][kw] = face_blend(gl.f[c][kw], gh.f[c][kw], t);
        }
    }
}

// rk3_kernel (SC:1553-1611) on interior cells, then enforce_admissible_kernel (SC:918-958) and
// cons_to_prim_kernel (SC:840-864) + al_prim copy on every cell, then the dt candidate of
// timestep_kernel (SC:1686-1705) -- each step selected by `flags`.
// Returns the bit pattern of the cell's time-step candidate (all ones when it has none).
// Binary32 pre-check of the combine's admissibility tests (both forms): true only when the
// binary64 state Q certainly has finite components, partial densities at or above the 1e-10 floor,
// alpha inside [1e-8, 1 - 1e-8] (so neither alpha clamp acts) and no energy repair
// ((E - kin)(1 + Gamma) - Pi >= 1e-8 (1 + Gamma), enforce_admissible_kernel SC:918-958). Rounding
// Q to binary32 moves each component by at most 2^-24 of it; the repair test's binary32 value is
// within about 10 roundings (6e-7) of its magnitude, and the test demands 4e-6 of it. A true
// result lets the caller skip those binary64 tests, whose outcome it has proved; the results are
// the same bits.
__device__ __forceinline__ bool cell_surely_admissible(const Eos &e, const double *Q)
{
    const float m1 = to_f32(Q[0]), m2 = to_f32(Q[1]), mx = to_f32(Q[2]), my = to_f32(Q[3]);
    const float E = to_f32(Q[4]), a = to_f32(Q[5]);
    if (!(isfinite(m1) && isfinite(m2) && isfinite(mx) && isfinite(my) && isfinite(E) && isfinite(a)))
        return false;
    const float lo = float(kPpRho) * 1.000001f;
    if (!(m1 >= lo && m2 >= lo)) return false;
    if (!(a >= float(kPrimAlphaFloor) * 1.000001f && 1.0f - a >= 5.0e-8f)) return false;
    const float rho = m1 + m2, kin = 0.5f * (mx * mx + my * my) / rho;
    const float a2 = 1.0f - a, gb = a * e.r1f + a2 * e.r2f, pb = a * e.k1f + a2 * e.k2f;
    const float gp1 = 1.0f + gb;
    const float v = (E - kin) * gp1 - pb - float(kPpCtilde) * gp1;
    const float mag = (fabsf(E) + kin) * gp1 + fabsf(pb) + float(kPpCtilde) * gp1;
    return v > 4.0e-6f * mag;
}

// 1 / (rho Gamma) of the primitive recovery, both forms: the Newton-Raphson reciprocal iteration
// y <- y + y (1 - x y) in binary64 (residual and update each one fused multiply-add; e.g. Muller et
// al., Handbook of Floating-Point Arithmetic, ch. 5), seeded with the binary32 reciprocal of x
// rounded to binary32 (relative error below 2^-23). Two steps square that to below 2^-92 before
// their own roundings, so the result is within about one unit in the last place of the quotient --
// binary64 accuracy for the accumulation, without the division's longer binary64 sequence. Outside
// binary32's normal range it divides. One form for every instantiation of the combine, so the
// closures (which run the binary64 one for both forms) and the fused stage give the same bits.
__device__ __forceinline__ double recovery_recip(double x)
{
    const float xf = to_f32(x), af = fabsf(xf);
    if (!(af >= 1.0e-37f && af <= 1.0e37f)) return 1.0 / x;
    double y = to_f64(__frcp_rn(xf));
    double r = __fma_rn(-x, y, 1.0);
    y = __fma_rn(y, r, y);
    r = __fma_rn(-x, y, 1.0);
    return __fma_rn(y, r, y);
}

// NP: limiter passes whose blends are deferred (3 in the fused stage: the limited fluxes are rebuilt
// from fh/gh, fl/gl and the three theta arrays; 0 when fh/gh already hold them).
template <typename FT, int NP = 0>
__device__ __forceinline__ unsigned long long final_body(const Grid &g, const Eos &e, unsigned flags,
                                                         const Fields &q, const Fields &old,
                                                         const Face<FT> &fh, const Face<FT> &gh,
                                                         const Face<FT> &fl, const Face<FT> &gl,
                                                         FT *const theta[3],
                                                         double dt, const double *dt_dev,
                                                         double alpha, double beta,
                                                         const Counters &cnt, int i, int j)
{
    bool inb = i < g.nxg && j < g.nyg;
    bool interior = inb && i >= g.g && i < g.g + g.nx && j >= g.g && j < g.g + g.ny;
    unsigned long long dt_bits = ~0ull;
    if (inb && (interior || (flags & (FIN_ADMISSIBLE | FIN_PRIM)))) {
        long long kf = kf_of(q, i, j);
        double Q[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) Q[c] = q.f[c][kf];
        bool wrote_q = false;
        if (interior && (flags & FIN_SAVE_OLD)) {
            long long ko = (long long)i * old.pitch + j;
#pragma unroll
            for (int c = 0; c < 6; ++c) old.f[c][ko] = Q[c];
        }
        if (interior && (flags & FIN_RK3)) {
            if (dt_dev) dt = *dt_dev;
            const CellFaces<FT, NP> cf(g, theta, i, j);
            const FT idx = cst<FT>(g.inv_dx, g.inv_dxf), idy = cst<FT>(g.inv_dy, g.inv_dyf);
            FT ap;
            if constexpr (sizeof(FT) == 4) ap = to_f32(q.f[F_ALP][kf]);
            else ap = q.f[F_ALP][kf];
            FT res[6];
#pragma unroll
            for (int c = 0; c < 5; ++c)
                res[c] = div_sum(cf.xp(fh, fl, c) - cf.xm(fh, fl, c), idx, cf.yp(gh, gl, c) - cf.ym(gh, gl, c), idy);
            FT src6x = src_term(ap, cf.xp(fh, fl, 6) - cf.xm(fh, fl, 6), idx);
            FT src6y = src_term(ap, cf.yp(gh, gl, 6) - cf.ym(gh, gl, 6), idy);
            res[5] = div_sum(cf.xp(fh, fl, 5) - cf.xm(fh, fl, 5), idx, cf.yp(gh, gl, 5) - cf.ym(gh, gl, 5), idy) -
                     src6x - src6y;
            long long ko = (long long)i * old.pitch + j;
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                double rc;
                if constexpr (sizeof(FT) == 4) rc = to_f64(res[c]);
                else rc = res[c];
                double base = __fma_rn(-dt, rc, Q[c]);
                if (!same_bits(beta, 1.0)) base = __dmul_rn(beta, base);  // 1 * x is x: stage 1 skips it
                Q[c] = (flags & FIN_OLD_READ) ? __fma_rn(alpha, old.f[c][ko], base) : base;
            }
            wrote_q = true;
        }
        // 1/(rho Gamma) of the admissibility check, reused by the primitive recovery when alpha
        // is unchanged by the second clamp
        double rg_a1 = -1.0, rg_rho = 0.0, rg_inv = 0.0, rg_gb = 0.0, rg_pb = 0.0;
        // A binary32 pre-check proves most cells need no clamp, floor, NaN handling or repair;
        // they skip those binary64 tests (the recovery is unchanged)
        bool fast = false;
        if ((flags & FIN_ADMISSIBLE) && (flags & FIN_PRIM) && !(flags & FIN_EXACT_CHECKS))
            fast = cell_surely_admissible(e, Q);
        if ((flags & FIN_ADMISSIBLE) && fast) {
            const double a1 = Q[F_AL], rho = Q[0] + Q[1];
            double gb, pb;
            mix_gamma_pibig(e, a1, gb, pb);
            rg_a1 = a1; rg_rho = rho; rg_inv = recovery_recip(rho * gb); rg_gb = gb; rg_pb = pb;
            wrote_q = true;
        } else if (flags & FIN_ADMISSIBLE) {
            double a1 = clamp01_pp(Q[F_AL]);
            double m1 = Q[0], m2 = Q[1], mx = Q[2], my = Q[3], E = Q[4];
            bool nonfinite = isnan(m1) || isnan(m2) || isnan(mx) || isnan(my) || isnan(E);
            if (isnan(m1) || m1 < kPpRho) m1 = kPpRho;
            if (isnan(m2) || m2 < kPpRho) m2 = kPpRho;
            if (isnan(mx)) mx = 0.0;
            if (isnan(my)) my = 0.0;
            double rho = m1 + m2;
            double gb, pb;
            mix_gamma_pibig(e, a1, gb, pb);
            const double inv = recovery_recip(rho * gb);
            const double ir = gb * inv;
            double uu = mx * ir, vv = my * ir;
            double kin = 0.5 * rho * (uu * uu + vv * vv);
            double p = (E - pb - kin) * (rho * inv);
            // E - kin - p_inf < floor with p_inf = Pi / (1 + Gamma), multiplied by 1 + Gamma > 0
            const double gp1 = 1.0 + gb;
            bool repair = isnan(E) || isnan(p) || ((E - kin) * gp1 - pb < kPpCtilde * gp1);
            if (repair) {
                double gg, pi;
                mix_gamma_pinf(e, a1, gg, pi);
                double p_min = kPpCtilde * (gg - 1.0) - pi;
                E = gb * p_min + pb + kin;
            }
            rg_a1 = a1; rg_rho = rho; rg_inv = inv; rg_gb = gb; rg_pb = pb;
            Q[0] = m1;
            Q[1] = m2;
            Q[2] = mx;
            Q[3] = my;
            Q[4] = E;
            Q[5] = a1;
            wrote_q = true;
            if (cnt.repaired) {
                count_if(cnt.repaired, repair);
                count_if(cnt.nonfinite, nonfinite);
            }
        }
        if (flags & FIN_PRIM) {
            double a1 = Q[F_AL];
            if (!fast) {
                if (a1 < kPrimAlphaFloor) a1 = kPrimAlphaFloor;
                if (a1 > 1.0 - kPrimAlphaFloor) a1 = 1.0 - kPrimAlphaFloor;
            }
            Q[F_AL] = a1;
            // the admissibility block's density is Q[0] + Q[1] of the state as it left it
            const double rho = (flags & FIN_ADMISSIBLE) ? rg_rho : Q[0] + Q[1];
            double gb, pb, inv;
            if (fast || (a1 == rg_a1 && rho == rg_rho)) {
                gb = rg_gb; pb = rg_pb; inv = rg_inv;
            } else {
                mix_gamma_pibig(e, a1, gb, pb);
                inv = recovery_recip(rho * gb);
            }
            double ir = gb * inv;
            double uu = Q[2] * ir, vv = Q[3] * ir;
            double pp = (Q[4] - pb - 0.5 * rho * (uu * uu + vv * vv)) * (rho * inv);
            q.f[F_U][kf] = uu;
            q.f[F_V][kf] = vv;
            q.f[F_P][kf] = pp;
            q.f[F_ALP][kf] = a1;
            q.f[F_AL][kf] = a1;
            if (interior && (flags & FIN_DT)) {
                if constexpr (sizeof(FT) == 4) {
                    // Precision form: c^2 = ((1 + Gamma) p + Pi) / (Gamma rho), the numerator (which
                    // cancels for p near -p_inf) in binary64, the rest of the CFL candidate in
                    // binary32 with one division: sx sy / (sx + sy) = dx dy / (dy a + dx b),
                    // a = |u| + c, b = |v| + c.
                    float c2 = to_f32(((1.0 + gb) * pp + pb) * inv);
                    if (c2 < float(kTiny)) c2 = float(kTiny);
                    const float c = sqrtf(c2);
                    const float a = fabsf(to_f32(uu)) + c, b = fabsf(to_f32(vv)) + c;
                    const float dxf = to_f32(g.dx), dyf = to_f32(g.dy);
                    const double d = to_f64((dxf * dyf) / (dyf * a + dxf * b));
                    dt_bits = (unsigned long long)__double_as_longlong(d);
                } else {
                    // timestep_kernel's sx sy / (sx + sy), sx = dx / (|u| + c), sy = dy / (|v| + c)
                    // (SC:1686-1705), as one quotient dx dy / (dy (|u| + c) + dx (|v| + c)), with
                    // the face sweep's sound speed and quotient
                    const double c = sound_speed_r<double, true>(e, ir, pp, a1);
                    const double d = div_nr(g.dx * g.dy, g.dy * (fabs(uu) + c) + g.dx * (fabs(vv) + c));
                    dt_bits = (unsigned long long)__double_as_longlong(d);
                }
            }
        }
        if (wrote_q) {
#pragma unroll
            for (int c = 0; c < 6; ++c) q.f[c][kf] = Q[c];
        }
    }
    return dt_bits;
}

// (num gb < kPpCtilde gp1) as binary64 evaluates it, for Gamma gb > 0 and gp1 = 1 + gb: the
// pressure-floor test of the first-order state below, num = (1 + Gamma) p + Pi. Decided from the
// binary32 roundings where the products are more than 2^-20 apart: each side is within 3 x 2^-24 of
// its binary64 value (two operand roundings and the product's; 1e-8f is within 2^-25 of 1e-8, a
// product below the normal range is off by 2^-150 against a right side above 1e-8), and a negative
// num is below at once. Elsewhere, and for operands outside [2^-100, 2^100], binary64 decides.
__device__ __forceinline__ bool below_floor(double num, double gb, double gp1)
{
    const float g = to_f32(gb), h = to_f32(gp1);
    if (g >= 0x1p-100f && g <= 0x1p100f && h <= 0x1p100f) {
        const float lhs = to_f32(num) * g, rhs = float(kPpCtilde) * h;
        if (lhs > rhs * (1.0f + 0x1p-20f)) return false;
        if (lhs < rhs * (1.0f - 0x1p-20f)) return true;
    }
    return num * gb < kPpCtilde * gp1;
}

// Binary32 copies of the cell state for the face sweep, the entropy in binary32, and the
// first-order HLLC cell state whose pressure floor and the numerator of its sound speed are
// recovered in binary64 (the stiffened-gas p + p_inf cancels to round-off of p_inf ~ 6e8 in
// binary32).
__device__ __forceinline__ void prep32_body(const Grid &g, const Eos &e, const Fields &q, const PrepT<float> &p, const Cells32 &c, bool sw64,
                                            bool prechecks, int i, int j)
{
    long long kf = kf_of(q, i, j), kw = kw_of(g, i, j);
    const double ar1 = q.f[F_AR1][kf], ar2 = q.f[F_AR2][kf], ru = q.f[F_RU][kf], rv = q.f[F_RV][kf];
    const double pp = q.f[F_P][kf], al = q.f[F_AL][kf];
    const float ar1f = to_f32(ar1), ar2f = to_f32(ar2), ruf = to_f32(ru), rvf = to_f32(rv);
    const float pf = to_f32(pp), alf = to_f32(al);
    c.ar1[kw] = ar1f;
    c.ar2[kw] = ar2f;
    c.ru[kw] = ruf;
    c.rv[kw] = rvf;
    c.p[kw] = pf;
    c.al[kw] = alf;
    c.u[kw] = to_f32(q.f[F_U][kf]);
    c.v[kw] = to_f32(q.f[F_V][kf]);
    c.E[kw] = to_f32(q.f[F_E][kf]);

    double gb, pb;  // Gamma and Pi of the cell's own fraction
    mix_gamma_pibig(e, al, gb, pb);
    double gp1 = 1.0 + gb;
    const double rho = ar1 + ar2;
    if (sw64) {  // binary64 switches: the entropy of the binary64 form (ent32 is the ent array)
        double ge, pie;
        mix_from_gp1<double, true>(gb, gp1, pb, ge, pie);  // entropy_gamma, 1 + Gamma at hand
        store_entropy_r(p, kw, ge, rho, pp, prechecks);
    } else {
        float ge, pie;
        mix_gamma_pinf(e, alf, ge, pie);
        float rho_e = ar1f + ar2f;
        if (rho_e < float(kTiny)) rho_e = float(kTiny);
        p.ent[kw] = pf / powf(rho_e, ge);
    }

    // With g = 1 + 1/Gamma and p_inf = Pi / (1 + Gamma): (p + p_inf) / (g - 1) < floor  <=>
    // ((1 + Gamma) p + Pi) Gamma < floor (1 + Gamma), and c^2 = ((1 + Gamma) p + Pi) / (Gamma rho).
    double a = al;
    if (!alpha_inside(al)) {  // a clamped fraction: its own mixture
        a = clamp01_pp(al);
        mix_gamma_pibig(e, a, gb, pb);
        gp1 = 1.0 + gb;
    }
    double pl = pp;
    // the numerator cancels for p near -p_inf and stays binary64; the quotient and root do not
    double num = gp1 * pl + pb;
    if (wisnan(pl) || below_floor(num, gb, gp1)) {
        double gg, pi;
        mix_gamma_pinf(e, a, gg, pi);
        pl = kPpCtilde * (gg - 1.0) - pi;
        num = gp1 * pl + pb;
    }
    const float rhof = ar1f + ar2f;
    float val = to_f32(num) / (to_f32(gb) * to_f32(rho));
    if (val < float(kTiny)) val = float(kTiny);
    const float irf = 1.0f / rhof;
    const float u = ruf * irf, v = rvf * irf;
    const float af = to_f32(a), plf = to_f32(pl);
    p.lu[kw] = u;
    p.lv[kw] = v;
    p.lp[kw] = plf;
    p.la[kw] = af;
    p.lc[kw] = sqrtf(val);
    p.lE[kw] = prim_to_energy(e, rhof, u, v, plf, af);
}

// Smoothness indicators and Ducros sensor in binary32 (sensor_kernel's arithmetic).
__device__ __forceinline__ void sensor32_body(const Grid &g, const Eos &e, const Fields &q, const PrepT<float> &p,
                                              const Cells32 &c, int sc, bool sw64, bool prechecks, int i, int j)
{
    long long kw = kw_of(g, i, j);
    const long long W = g.nyg;
    if (sw64) {  // the binary64 sensors, stored as their side of the sweep's thresholds
        const long long kf = kf_of(q, i, j);
        if (i >= 2 && i < g.nxg - 2) p.cx[kw] = thinc_side(e, q, p, kw, kf, W, q.pitch, prechecks);
        if (j >= 2 && j < g.nyg - 2) p.cy[kw] = thinc_side(e, q, p, kw, kf, 1, 1, prechecks);
        if (!sc) return;
        if (i < 2 || i >= g.nxg - 2 || j < 2 || j >= g.nyg - 2) {
            p.sx[kw] = side_of(1.0, kSigmaSmooth);
            p.sy[kw] = side_of(1.0, kSigmaSmooth);
            return;
        }
        if (prechecks) {  // the pre-check reads prep's binary32 copies (to_f32 of the state)
            ducros_sides_pre(q, i, j, c.u, c.v, c.p, kw, W, 1, p.sx[kw], p.sy[kw]);
        } else {
            double sx, sy;
            ducros_xy(q, i, j, sx, sy);
            p.sx[kw] = side_of(sx, kSigmaSmooth);
            p.sy[kw] = side_of(sy, kSigmaSmooth);
        }
        return;
    }
    const float *en = p.ent;
    if (i >= 2 && i < g.nxg - 2)
        p.cx[kw] = cator2_val(en[kw - 2 * W], en[kw - W], en[kw], en[kw + W], en[kw + 2 * W]);
    if (j >= 2 && j < g.nyg - 2)
        p.cy[kw] = cator2_val(en[kw - 2], en[kw - 1], en[kw], en[kw + 1], en[kw + 2]);
    if (!sc) return;
    if (i < 2 || i >= g.nxg - 2 || j < 2 || j >= g.nyg - 2) {
        p.sx[kw] = 1.0f;
        p.sy[kw] = 1.0f;
        return;
    }
    const float *U = c.u, *V = c.v, *P = c.p;
    float der_ux = 0.5f * (-U[kw - W] + U[kw + W]);
    float der_vx = 0.5f * (-V[kw - W] + V[kw + W]);
    float der_uy = 0.5f * (-U[kw - 1] + U[kw + 1]);
    float der_vy = 0.5f * (-V[kw - 1] + V[kw + 1]);
    float div_u = der_ux + der_vy;
    float curl_u = der_vx - der_uy;
    float ducros = div_u * div_u / (div_u * div_u + curl_u * curl_u + 1.0e-30f);
    float p0 = P[kw];
    float pm2 = P[kw - 2 * W], pm1 = P[kw - W], pp1 = P[kw + W], pp2 = P[kw + 2 * W];
    float aa = fabsf(-pm2 + 16.0f * pm1 - 30.0f * p0 + 16.0f * pp1 - pp2);
    float bb = fabsf(pm2 + 16.0f * pm1 + 30.0f * p0 + 16.0f * pp1 + pp2);
    p.sx[kw] = (aa / (bb + 1.0e-30f)) * ducros;
    pm2 = P[kw - 2];
    pm1 = P[kw - 1];
    pp1 = P[kw + 1];
    pp2 = P[kw + 2];
    aa = fabsf(-pm2 + 16.0f * pm1 - 30.0f * p0 + 16.0f * pp1 - pp2);
    bb = fabsf(pm2 + 16.0f * pm1 + 30.0f * p0 + 16.0f * pp1 + pp2);
    p.sy[kw] = (aa / (bb + 1.0e-30f)) * ducros;
}

// Cell-state sources of the sweep: the caller's binary64 arrays (row pitch of the fields) or the
// binary32 copies in the workspace (row pitch of the padded grid).
struct Src64 {
    Fields q;
    __device__ __forceinline__ long long pitch() const { return q.pitch; }
    __device__ __forceinline__ void load(long long k, double u[6]) const
    {
        u[0] = q.f[F_AR1][k]; u[1] = q.f[F_AR2][k]; u[2] = q.f[F_RU][k];
        u[3] = q.f[F_RV][k]; u[4] = q.f[F_P][k]; u[5] = q.f[F_AL][k];
    }
};
struct Src32 {
    Cells32 c;
    long long nyg;
    __device__ __forceinline__ long long pitch() const { return nyg; }
    __device__ __forceinline__ void load(long long k, float u[6]) const
    {
        u[0] = c.ar1[k]; u[1] = c.ar2[k]; u[2] = c.ru[k];
        u[3] = c.rv[k]; u[4] = c.p[k]; u[5] = c.al[k];
    }
};

// Where a face body reads its inputs: the six fields of the cells at offsets -2..3 along the sweep
// from the face's cell 0, the first-order cell states (normal and tangential velocity, floored
// pressure, clamped alpha, sound speed, energy) of cells 0 and 1, and the two sensors of cells
// -1..2. GlobalView reads the arrays; SmemView (wm_faces.cu) reads a block's staged tile. Both give
// the same values, so a face's result does not depend on the view.
template <int DIR, typename T, typename CS>
struct GlobalView {
    CS cs;
    PrepT<T> p;
    long long kf, kw, sf, sw;
    __device__ __forceinline__ GlobalView(const Grid &g, const CS &cs_, const PrepT<T> &p_, int i, int j)
        : cs(cs_), p(p_)
    {
        sf = DIR == 0 ? cs.pitch() : 1;
        sw = DIR == 0 ? g.nyg : 1;
        kf = (long long)i * cs.pitch() + j;
        kw = (long long)i * g.nyg + j;
    }
    __device__ __forceinline__ void cell(int o, T u[6]) const { cs.load(kf + o * sf, u); }
    __device__ __forceinline__ T un(int o) const { return (DIR == 0 ? p.lu : p.lv)[kw + o * sw]; }
    __device__ __forceinline__ T ut(int o) const { return (DIR == 0 ? p.lv : p.lu)[kw + o * sw]; }
    __device__ __forceinline__ T lp(int o) const { return p.lp[kw + o * sw]; }
    __device__ __forceinline__ T la(int o) const { return p.la[kw + o * sw]; }
    __device__ __forceinline__ T lc(int o) const { return p.lc[kw + o * sw]; }
    __device__ __forceinline__ T lE(int o) const { return p.lE[kw + o * sw]; }
    __device__ __forceinline__ T sens_c(int o) const { return (DIR == 0 ? p.cx : p.cy)[kw + o * sw]; }
    __device__ __forceinline__ T sens_s(int o) const { return (DIR == 0 ? p.sx : p.sy)[kw + o * sw]; }
};

// One face of the sweep in direction DIR: the face between cell (i, j) and its neighbour at +1
// along the sweep. Callers guarantee that the face exists. OD: the first-order values may be left to
// their consumers (Face::src.on), only their finiteness byte written.
template <int DIR, int VAR, int REC, typename T, bool OD = false, typename V, typename FT>
__device__ __forceinline__ void face_body(const Eos &e, const V &v, const Face<FT> &hi, const Face<FT> &lo,
                                          bool do_high, bool do_low, long long kw)
{
    constexpr int N = DIR == 0 ? 2 : 3;   // normal momentum field
    constexpr int TG = DIR == 0 ? 3 : 2;  // tangential momentum field

    // Cells 0 and 1 of the face (i and i+1 along the sweep).
    T U0[6], U1[6];
    v.cell(0, U0);
    v.cell(1, U1);

    if (do_low) {  // first-order HLLC of the two cell states (fx_low_kernel, SC:1303-1347)
        Side<T> L, R;
        first_order_side(U0[0], U0[1], v.un(0), v.ut(0), v.lp(0), v.la(0), v.lc(0), v.lE(0), L);
        first_order_side(U1[0], U1[1], v.un(1), v.ut(1), v.lp(1), v.la(1), v.lc(1), v.lE(1), R);
        bool done = false;
        if constexpr (OD && sizeof(T) == 8 && sizeof(FT) == 8) {
            if (lo.src.on) {
                // binary64 fused stage: the values are formed on demand where the limiter reads
                // them; here only their finiteness byte -- proved from the speeds where it can be
                // (nearly every face), else from the values themselves: the same byte either way
                T SL, SR, SP;
                hllc_speeds(L, R, SL, SR, SP);
                bool fin = hllc_surely_finite(L, R, SL, SR, SP);
                if (!fin) {
                    T f[6], us;
                    hllc<DIR>(L, R, f, us);
                    fin = finite_bits(FT(us));
#pragma unroll
                    for (int c = 0; c < 6; ++c) fin = fin && finite_bits(FT(f[c]));
                }
                lo.fin[kw] = fin ? 1 : 0;
                done = true;
            }
        }
        if (!done) {
            T f[6], us;
            hllc<DIR>(L, R, f, us);
            bool fin = finite_bits(FT(us));
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                lo.f[c][kw] = FT(f[c]);
                fin = fin && finite_bits(FT(f[c]));
            }
            lo.f[6][kw] = FT(us);
            if constexpr (sizeof(FT) == 8) lo.fin[kw] = fin ? 1 : 0;  // read by the binary64 limiter
        }
    }
    if (!do_high) return;

    // --- sensors (per-cell, computed by sensor_kernel) -------------------------------------------
    const T c_m1 = v.sens_c(-1), c_0 = v.sens_c(0), c_p1 = v.sens_c(1), c_p2 = v.sens_c(2);
    const bool use_thinc = flt(wmin(wmin(c_m1, c_0), wmin(c_p1, c_p2)), T(kThincThresh));
    bool smooth = false;
    if (VAR == kSC) {
        const T smax = wmax(wmax(v.sens_s(-1), v.sens_s(0)), wmax(v.sens_s(1), v.sens_s(2)));
        smooth = flt(smax, T(kSigmaSmooth));
    }

    // --- face-averaged state and eigenvector basis (SC:1039-1048) ------------------------------
    const T ar1a = half_of(U0[0] + U1[0]);
    const T ar2a = half_of(U0[1] + U1[1]);
    const T a1a = half_of(U0[5] + U1[5]);
    const T pa = half_of(U0[4] + U1[4]);
    const T rhoa = ar1a + ar2a;
    const T irhoa = sw_rcp(rhoa);
    FaceBasis<T> b;
    b.u = half_of(U0[2] + U1[2]) * irhoa;
    b.v = half_of(U0[3] + U1[3]) * irhoa;
    const T ca = sound_speed_r<T, true>(e, irhoa, pa, a1a);
    {
        const T ic = sw_rcp(ca);
        b.c = ca;
        b.c2 = ca * ca;
        b.inv2c = half_of(ic);
        b.inv2c2 = half_of(ic * ic);
        b.Y1 = ar1a * irhoa;
        b.Y2 = ar2a * irhoa;
        b.Y1c2 = b.Y1 * (ic * ic);
        b.Y2c2 = b.Y2 * (ic * ic);
    }

    // --- characteristic projection of cells -2..3 (MUSCL needs -1..2) --------------------------
    constexpr int O0 = REC == kMp5 ? 0 : 1, O1 = REC == kMp5 ? 6 : 5;
    T W[6][6];
#pragma unroll
    for (int o = O0; o < O1; ++o) {
        T u[6];
        if (o == 2) {
#pragma unroll
            for (int f = 0; f < 6; ++f) u[f] = U0[f];
        } else if (o == 3) {
#pragma unroll
            for (int f = 0; f < 6; ++f) u[f] = U1[f];
        } else {
            v.cell(o - 2, u);
        }
        S6<T> w = to_char<DIR>(b, u);
#pragma unroll
        for (int f = 0; f < 6; ++f) W[o][f] = w.v[f];
    }

    // --- reconstruction (SC:1062-1092; M10:958-979) ---------------------------------------------
    T wL[6], wR[6];
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        const bool thinc_f = (f == 1 || f == 2) ? use_thinc : (f == 4 ? (VAR == kM10 || use_thinc) : false);
        const bool central_f = VAR == kSC && f == 3 && smooth;
        if (thinc_f) {
            wL[f] = thinc_ul(e, W[1][f], W[2][f], W[3][f]);
            wR[f] = thinc_ur(e, W[2][f], W[3][f], W[4][f]);
        } else if (central_f) {
            T iph = REC == kMp5 ? central6_avg(W[0][3], W[1][3], W[2][3], W[3][3], W[4][3], W[5][3])
                                : central4(W[1][3], W[2][3], W[3][3], W[4][3]);
            wL[f] = iph;
            wR[f] = iph;
        } else if (REC == kMp5) {
            if constexpr (sizeof(T) == 8) {  // difference form, the differences shared by both values
                const T d0 = W[1][f] - W[0][f], d1 = W[2][f] - W[1][f], d2 = W[3][f] - W[2][f];
                const T d3 = W[4][f] - W[3][f], d4 = W[5][f] - W[4][f];
                wL[f] = mp5_diff(W[2][f], W[3][f], d0, d1, d2, d3);
                wR[f] = mp5_diff(W[3][f], W[2][f], -d4, -d3, -d2, -d1);
            } else {
                wL[f] = mp5_ul(W[0][f], W[1][f], W[2][f], W[3][f], W[4][f]);
                wR[f] = mp5_ur(W[1][f], W[2][f], W[3][f], W[4][f], W[5][f]);
            }
        } else {
            wL[f] = muscl_char_ul(W[1][f], W[2][f], W[3][f]);
            wR[f] = muscl_char_ur(W[2][f], W[3][f], W[4][f]);
        }
    }

    // --- back-projection and positivity fallback (SC:1095-1115; M10:1000-1025) ----------------
    S6<T> phL = to_phys<DIR>(b, wL), phR = to_phys<DIR>(b, wR);
    if (VAR == kM10) {
        const S6<T> phfL = to_phys<DIR>(b, W[2]), phfR = to_phys<DIR>(b, W[3]);
        phL = pp_limit_reconstructed_state(e, phL, phfL);
        phR = pp_limit_reconstructed_state(e, phR, phfR);
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            S6<T> &ph = s == 0 ? phL : phR;
            const S6<T> &pf = s == 0 ? phfL : phfR;
            if (!fge(ph.v[0], T(0))) ph.v[0] = pf.v[0];  // x < 0 or NaN
            if (!fge(ph.v[1], T(0))) ph.v[1] = pf.v[1];
            if (flt(ph.v[5], T(0)) || fgt(ph.v[5], T(1))) ph.v[5] = pf.v[5];
            if (flt(rho_ctilde2_sc(e, ph), T(kPpCtilde)) || wisnan(ph.v[4])) ph.v[4] = pf.v[4];
            ph = pp_floor_pressure_state(e, ph);
        }
        if (!fge(ca, T(0))) {  // ca < 0 or NaN
            phL = phfL;
            phR = phfR;
        }
    } else {
        // The same fallbacks; the first-order state (the back-projection of cell 0 or 1) is formed
        // only for a side that needs one of its components.
        const bool bad_ca = !fge(ca, T(0));  // ca < 0 or NaN: both sides take it whole
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            S6<T> &ph = s == 0 ? phL : phR;
            const bool b0 = !fge(ph.v[0], T(0)), b1 = !fge(ph.v[1], T(0));  // x < 0 or NaN
            const bool b5 = flt(ph.v[5], T(0)) || fgt(ph.v[5], T(1)), b4 = wisnan(ph.v[4]);
            if (bad_ca || b0 || b1 || b4 || b5) {
                const S6<T> pf = to_phys<DIR>(b, s == 0 ? W[2] : W[3]);
                if (bad_ca) {
                    ph = pf;
                } else {
                    if (b0) ph.v[0] = pf.v[0];
                    if (b1) ph.v[1] = pf.v[1];
                    if (b5) ph.v[5] = pf.v[5];
                    if (b4) ph.v[4] = pf.v[4];
                }
            }
        }
    }

    // --- HLLC on the reconstructed states (SC:1118-1133) ---------------------------------------
    Side<T> S[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const S6<T> &ph = s == 0 ? phL : phR;
        Side<T> &d = S[s];
        d.ar1 = ph.v[0];
        d.ar2 = ph.v[1];
        d.rho = ph.v[0] + ph.v[1];
        const T ir = sw_rcp(d.rho);
        d.un = ph.v[N] * ir;
        d.ut = ph.v[TG] * ir;
        d.p = ph.v[4];
        d.a = ph.v[5];
        d.c = sound_speed_r<T, true>(e, ir, d.p, d.a);
        if constexpr (sizeof(T) == 8) {  // hllc forms the energy of the side it reads
            mix_gamma_pibig(e, d.a, d.gb, d.pb);
            d.E = T(0);
        } else {
            d.E = prim_to_energy(e, d.rho, d.un, d.ut, d.p, d.a);
        }
    }
    T f[6], us;
    hllc<DIR, sizeof(T) == 8>(S[0], S[1], f, us);
#pragma unroll
    for (int c = 0; c < 6; ++c) hi.f[c][kw] = FT(f[c]);
    hi.f[6][kw] = FT(us);
}

}  // namespace wm
