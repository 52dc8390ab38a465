// wm_device.cuh -- device functions of the per-stage RHS (sm_103a).
//
// Each function states the reference device function it computes (SC = sainath_SC_it_works.py).
// They are templated on the arithmetic type T of the face sweeps: double for the plain form,
// float for the bulk of the precision form. Branch structure, thresholds and the order of the
// operations that decide branches follow the reference; divisions by run-time constants are
// replaced by multiplications with host-computed reciprocals, and divisions by the same value are
// shared (a relative difference of a few ulp, far inside the 1e-10 parity tolerance).
#pragma once
#include <cmath>
#include <cuda_runtime.h>
#include <stdint.h>

namespace wm {

// ------------------------------------------------------------------------------------------------
// Launch-constant parameter blocks (passed by value as kernel arguments).
// ------------------------------------------------------------------------------------------------
struct Eos {
    double g1, p1, g2, p2;  // gamma, p_inf of fluid 1 and 2
    double r1, r2;          // 1/(g1-1), 1/(g2-1)
    double k1, k2;          // g1*p1/(g1-1), g2*p2/(g2-1)
    double dr, dk;          // r1 - r2, k1 - k2 (the mixture's slopes in alpha1)
    double thinc_t1;        // tanh(beta/2), beta = 1.8 (computed once on the host)
    double thinc_inv_t1;    // 1/tanh(beta/2)
    float r1f, r2f, k1f, k2f, drf, dkf;  // binary32 copies (binary32 kernels use these: no conversion on the
    float thinc_t1f, thinc_inv_t1f;  // device, where it would issue on the narrow binary64 pipe)
};

// The run's constants of the stiffened-gas mixture (host side).
inline Eos make_eos(double g1, double p1, double g2, double p2)
{
    Eos E;
    E.g1 = g1; E.p1 = p1; E.g2 = g2; E.p2 = p2;
    E.r1 = 1.0 / (g1 - 1.0); E.r2 = 1.0 / (g2 - 1.0);
    E.k1 = g1 * p1 / (g1 - 1.0); E.k2 = g2 * p2 / (g2 - 1.0);
    E.thinc_t1 = std::tanh(1.8 * 0.5);
    E.thinc_inv_t1 = 1.0 / E.thinc_t1;
    E.dr = E.r1 - E.r2; E.dk = E.k1 - E.k2;
    E.r1f = float(E.r1); E.r2f = float(E.r2); E.k1f = float(E.k1); E.k2f = float(E.k2);
    E.drf = float(E.dr); E.dkf = float(E.dk);
    E.thinc_t1f = float(E.thinc_t1); E.thinc_inv_t1f = float(E.thinc_inv_t1);
    return E;
}

// A run-time constant in the arithmetic type T: the binary64 value, or its host-made binary32 copy.
template <typename T> __device__ __forceinline__ T cst(double d, float f);
template <> __device__ __forceinline__ double cst<double>(double d, float) { return d; }
template <> __device__ __forceinline__ float cst<float>(double, float f) { return f; }

struct Grid {
    int nx, ny, g;       // interior size and ghost width
    int nxg, nyg;        // padded size
    long long pitch;     // elements between x rows
    double dx, dy, inv_dx, inv_dy, cfl;
    float inv_dxf, inv_dyf;  // binary32 copies of 1/dx, 1/dy
};

// Reference constants (SC:44-70).
constexpr double kTiny = 1.0e-20;
constexpr double kEpsM = 1.0e-20;
constexpr double kMp5Alpha = 4.0;
constexpr double kB2 = 4.0 / 3.0;
constexpr double kKappa = 1.0 / 3.0;
constexpr double k1o60 = 1.0 / 60.0;
constexpr double kYuxin = 0.9 * 0.35 * 1.0e-2 / (1.0 - 0.9 * 0.35);
constexpr double kThincThresh = 0.35;
constexpr double kPpRho = 1.0e-10;
constexpr double kPpAlpha = 1.0e-10;
constexpr double kPpCtilde = 1.0e-8;
constexpr double kPpHsRho = 1.0e-11;
constexpr double kPpHsAlpha = 1.0e-11;
constexpr double kPpHsCtilde = 1.0e-9;
constexpr double kSigmaSmooth = 0.01;
constexpr double kPrimAlphaFloor = 1.0e-8;  // cons_to_prim clamp (SC:852-853)

// Warp's float builtins: min/max as a<b?a:b / a>b?a:b; sign(x) = x<0 ? -1 : +1.
// binary64 <-> binary32 conversions on the integer pipe. GB300 issues the hardware conversions on
// its narrow binary64 pipe (about 17 clocks a warp); these take about 4. Both give the IEEE 754
// round-to-nearest-even result bit for bit: to_f32 keeps the top 23 fraction bits and rounds at bit
// 28 of the low word (ties to the even significand; a carry into the exponent is the correct
// rounding, up to infinity), to_f64 widens exactly; zeros, subnormals, results outside binary32's
// normal range, infinities and NaN take the hardware instruction. (Zero tests on the integer pipe --
// in C++ or PTX, in either direction -- were measured: each made the kernels that convert a state
// at rest slower, though it removed hardware conversions.)
__device__ __forceinline__ float to_f32(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7ffu);  // binary64 biased exponent
    if (e >= 897 && e <= 1150) {              // binary32 biased exponent e - 896 in [1, 254]
        const unsigned f = ((hi & 0xfffffu) << 3) | (lo >> 29);
        const unsigned r = lo & 0x1fffffffu;
        unsigned bits = (hi & 0x80000000u) | ((unsigned)(e - 896) << 23) | f;
        bits += (r > 0x10000000u || (r == 0x10000000u && (f & 1u))) ? 1u : 0u;
        return __uint_as_float(bits);
    }
    return __double2float_rn(x);
}
__device__ __forceinline__ double to_f64(float x)
{
    const unsigned b = __float_as_uint(x);
    const unsigned e = (b >> 23) & 0xffu;
    if (e != 0u && e != 0xffu) {
        const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
        return __hiloint2double((int)hi, (int)(b << 29));
    }
    return (double)x;
}

// x as the binary32 pair hi + lo on the integer pipe: hi = to_f32(x), lo = the binary32 rounding of
// x - hi. x - hi is exact in binary64: a signed multiple of x's last-place unit 2^(e - 1075) below
// 2^28 in magnitude, which x's low 29 significand bits and the rounding direction of hi give
// directly; its conversion (round to nearest) and the exact power-of-two scaling give the same bits
// as to_f32(x - hi) in binary64. Domain: binary64 exponent e in [949, 1150] (|x| in [2^-74, 2^128),
// every scaled remainder a normal binary32) -- there hi + lo is within 2^-48 |x| of x, unless hi
// rounded up to infinity; elsewhere lo = 0.
__device__ __forceinline__ void split32(double x, float &hi, float &lo)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
    const int e = (int)((hw >> 20) & 0x7ffu);
    hi = to_f32(x);
    lo = 0.0f;
    if (e >= 949 && e <= 1150) {
        const unsigned f = ((hw & 0xfffffu) << 3) | (lw >> 29);
        const int r = (int)(lw & 0x1fffffffu);
        const bool up = r > 0x10000000 || (r == 0x10000000 && (f & 1u));  // to_f32's rounding
        const int rem = up ? r - 0x20000000 : r;                           // |x| - |hi| in units
        // x - hi times 2^(e - 1075); a zero remainder gives +0, as x - hi does
        lo = __int2float_rn((hw >> 31) ? -rem : rem) * __int_as_float((e - 948) << 23);
    }
}

// log1p and expm1 of a binary32 x for the ratio pre-check: for |x| <= 2^-5 the Taylor series to the
// fifth power by Horner's rule with fused multiply-adds (truncation below 2^-27.5 relative, the
// last two roundings 2^-24 each: within 2^-22.9 of the exact value), elsewhere CUDA's log1pf /
// expm1f (within 1 ulp). In smooth flow the arguments are that small, and the series costs five
// operations.
__device__ __forceinline__ float log1p_pc(float x)
{
    if (!(fabsf(x) <= 0.03125f)) return log1pf(x);
    float t = __fmaf_rn(x, 0.2f, -0.25f);  // 1 - x/2 + x^2/3 - x^3/4 + x^4/5
    t = __fmaf_rn(x, t, 0.33333334f);
    t = __fmaf_rn(x, t, -0.5f);
    t = __fmaf_rn(x, t, 1.0f);
    return x * t;
}
__device__ __forceinline__ float expm1_pc(float x)
{
    if (!(fabsf(x) <= 0.03125f)) return expm1f(x);
    float t = __fmaf_rn(x, 0.008333334f, 0.041666668f);  // 1 + x/2 + x^2/6 + x^3/24 + x^4/120
    t = __fmaf_rn(x, t, 0.16666667f);
    t = __fmaf_rn(x, t, 0.5f);
    t = __fmaf_rn(x, t, 1.0f);
    return x * t;
}

// A binary64 result stored in the type T: to_f32 for binary32 storage (the same rounding as the
// implicit conversion, on the integer pipe), unchanged for binary64.
template <typename T> __device__ __forceinline__ T store_as(double x);
template <> __device__ __forceinline__ float store_as<float>(double x) { return to_f32(x); }
template <> __device__ __forceinline__ double store_as<double>(double x) { return x; }

// IEEE comparisons of binary64 values by integer compares of their bit patterns, off GB300's narrow
// binary64 pipe. Written in PTX: the same integer arithmetic in C++ is recognised by the compiler in
// some contexts and turned back into binary64 compares and min / max instructions (measured: 2-3
// binary64-pipe instructions for a minimum or a clamp written that way, 1 for the hardware compare,
// 0 for these).
// a < b: false when either operand is NaN; otherwise the order of the signed magnitudes
// k = sign ? -|bits| : |bits|, in which both zeros map to 0 (so -0 < +0 is false, as IEEE has it);
// a <= b likewise.
#define WM_DCMP_PTX(OP)                                                                                       \
    "{\n\t.reg .s64 ia, ib, ma, mb, na, nb;\n\t.reg .pred pa, pb, pc;\n\t"                                  \
    "mov.b64 ia, %1;\n\tmov.b64 ib, %2;\n\t"                                                                 \
    "and.b64 ma, ia, 0x7fffffffffffffff;\n\tand.b64 mb, ib, 0x7fffffffffffffff;\n\t"                          \
    "setp.lt.s64 pa, ia, 0;\n\tneg.s64 na, ma;\n\tselp.s64 na, na, ma, pa;\n\t"                              \
    "setp.lt.s64 pb, ib, 0;\n\tneg.s64 nb, mb;\n\tselp.s64 nb, nb, mb, pb;\n\t"                              \
    "setp.le.s64 pc, ma, 0x7ff0000000000000;\n\tsetp.le.and.s64 pc, mb, 0x7ff0000000000000, pc;\n\t"        \
    "setp." OP ".and.s64 pc, na, nb, pc;\n\tselp.u32 %0, 1, 0, pc;\n\t}"
__device__ __forceinline__ bool dlt(double a, double b)
{
    unsigned r;
    asm(WM_DCMP_PTX("lt") : "=r"(r) : "d"(a), "d"(b));
    return r != 0u;
}
__device__ __forceinline__ bool dle(double a, double b)
{
    unsigned r;
    asm(WM_DCMP_PTX("le") : "=r"(r) : "d"(a), "d"(b));
    return r != 0u;
}
#undef WM_DCMP_PTX
// x < 0: sign bit set, not a zero, not NaN
__device__ __forceinline__ bool dneg(double x)
{
    unsigned r;
    asm("{\n\t.reg .s64 ix, m;\n\t.reg .pred p;\n\tmov.b64 ix, %1;\n\t"
        "and.b64 m, ix, 0x7fffffffffffffff;\n\tsetp.lt.s64 p, ix, 0;\n\t"
        "setp.ne.and.s64 p, m, 0, p;\n\tsetp.le.and.s64 p, m, 0x7ff0000000000000, p;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r) : "d"(x));
    return r != 0u;
}
// x > 0: sign bit clear, not a zero, not NaN (as a signed integer: in (0, +inf])
__device__ __forceinline__ bool dpos(double x)
{
    unsigned r;
    asm("{\n\t.reg .s64 ix;\n\t.reg .pred p;\n\tmov.b64 ix, %1;\n\t"
        "setp.gt.s64 p, ix, 0;\n\tsetp.le.and.s64 p, ix, 0x7ff0000000000000, p;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r) : "d"(x));
    return r != 0u;
}

// IEEE comparisons in the arithmetic type T (binary64: the integer forms above, same results).
template <typename T> __device__ __forceinline__ bool flt(T a, T b) { return a < b; }
template <typename T> __device__ __forceinline__ bool fle(T a, T b) { return a <= b; }
template <> __device__ __forceinline__ bool flt<double>(double a, double b) { return dlt(a, b); }
template <> __device__ __forceinline__ bool fle<double>(double a, double b) { return dle(a, b); }
template <typename T> __device__ __forceinline__ bool fgt(T a, T b) { return flt(b, a); }
template <typename T> __device__ __forceinline__ bool fge(T a, T b) { return fle(b, a); }
template <typename T> __device__ __forceinline__ bool fpos(T x) { return x > T(0); }
template <> __device__ __forceinline__ bool fpos<double>(double x) { return dpos(x); }

// ------------------------------------------------------------------------------------------------
// Reciprocal, quotient and square root of the binary64 face sweep. GB300 issues binary64
// arithmetic on a narrow pipe (about two operations per SM per clock), where an IEEE division or
// square root is a chain of several dependent operations; the sweep is bound by that pipe. These
// forms take a binary32 seed from the integer pipe and the multi-function unit and refine it in
// binary64 with fused multiply-adds (Newton-Raphson and series refinement, and Markstein's
// residual correction of the quotient; e.g. Muller et al., Handbook of Floating-Point Arithmetic,
// ch. 5):
//   seed  s ~ 1/y: y truncated to 20 fraction bits (relative error < 2^-20), rcp.approx.f32
//         (<= 1 ulp), widened exactly, so e = 1 - y s has |e| < 2^-19.8;
//   rcp   s (1 + e + e^2) = 1/y (1 - e^3 / (1 - e)): relative error < 2^-59 before its own
//         roundings -- within one unit in the last place of 1/y (3 operations);
//   div   q0 = x s1, r = x - y q0 (one rounding), q = q0 + r s1: within about half a unit of x/y
//         (6 operations);
//   sqrt  h ~ 1/sqrt(x) from rsqrt.approx.f32 of x truncated (relative error < 2^-20.5),
//         z = x h, then twice z += (x - z^2) h/2 (the error goes 2^-20.5 -> 2^-40 -> < 2^-59):
//         within one unit of sqrt(x) (5 operations).
// Operands where the seed would not be a normal binary32 number or a product could leave the
// normal range -- zeros, subnormals, infinities, NaN, negative square-root operands, |y| (and the
// square-root operand) outside [2^-125, 2^125), |x| outside [2^-896, 2^897) -- take the IEEE
// operation, so special values give exactly what division and sqrt give. Elsewhere the results
// may differ from the correctly rounded ones by one unit in the last place (wm_check_sweep_arith
// counts any larger difference on random and boundary operands).
__device__ __forceinline__ double widen_normal(float f)  // exact, for a normal binary32 f
{
    const unsigned b = __float_as_uint(f);
    const unsigned hi = (b & 0x80000000u) | ((((b >> 23) & 0xffu) + 896u) << 20) | ((b & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(b << 29));
}
// y truncated to binary32 from its high word (sign, biased exponent ey in [898, 1147], 20 bits)
__device__ __forceinline__ float trunc_f32(unsigned hy, unsigned ey)
{
    return __uint_as_float((hy & 0x80000000u) | ((ey - 896u) << 23) | ((hy & 0xfffffu) << 3));
}
__device__ __forceinline__ unsigned exp_bits(unsigned hi) { return (hi >> 20) & 0x7ffu; }
__device__ __forceinline__ double rcp_refine(double y, unsigned hy, unsigned ey)
{
    float sf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(sf) : "f"(trunc_f32(hy, ey)));
    const double s = widen_normal(sf);
    const double e = __fma_rn(-y, s, 1.0);
    return __fma_rn(s, __fma_rn(e, e, e), s);
}
// The IEEE operations for the operands the seeded forms below leave to them (zeros, subnormals,
// infinities, NaN, out-of-range magnitudes), out of line, so that the compiler cannot evaluate
// them for every operand (as it did with the rare products of the exponent-arithmetic forms).
static __device__ __noinline__ double ieee_div_rare(double x, double y) { return x / y; }
static __device__ __noinline__ double ieee_sqrt_rare(double x) { return sqrt(x); }
__device__ __forceinline__ double rcp_nr(double y)
{
    const unsigned hy = (unsigned)__double2hiint(y), ey = exp_bits(hy);
    if (ey - 898u > 249u) return ieee_div_rare(1.0, y);
    return rcp_refine(y, hy, ey);
}
__device__ __forceinline__ double div_nr(double x, double y)
{
    const unsigned hy = (unsigned)__double2hiint(y), ey = exp_bits(hy);
    const unsigned ex = exp_bits((unsigned)__double2hiint(x));
    if (ey - 898u > 249u || ex - 127u > 1792u) return ieee_div_rare(x, y);
    const double s = rcp_refine(y, hy, ey);
    const double q0 = __dmul_rn(x, s);
    return __fma_rn(__fma_rn(-y, q0, x), s, q0);
}
__device__ __forceinline__ double sqrt_nr(double x)
{
    const unsigned hx = (unsigned)__double2hiint(x), ex = exp_bits(hx);
    if ((hx >> 31) || ex - 898u > 249u) return ieee_sqrt_rare(x);
    float hf;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(hf) : "f"(trunc_f32(hx, ex)));
    const double hh = widen_normal(0.5f * hf);  // h / 2, halved exactly in binary32
    double z = __dmul_rn(x, widen_normal(hf));
    z = __fma_rn(__fma_rn(-z, z, x), hh, z);
    return __fma_rn(__fma_rn(-z, z, x), hh, z);
}
// Two quotients a / b and c / d. Binary64: from one refined reciprocal of the product,
// a (d r) and c (b r) with r = rcp_nr(b d) -- 8 operations instead of 12, within a few units in the
// last place -- where b, d and b d lie in rcp_nr's seeded range and a, c in div_nr's (so every
// product stays normal); else, and in binary32, the two quotients.
__device__ __forceinline__ void div2_nr(double a, double b, double c, double d, double &q1, double &q2)
{
    const double bd = __dmul_rn(b, d);
    const unsigned e = exp_bits((unsigned)__double2hiint(bd));
    const unsigned eb = exp_bits((unsigned)__double2hiint(b)), ed = exp_bits((unsigned)__double2hiint(d));
    const unsigned ea = exp_bits((unsigned)__double2hiint(a)), ec = exp_bits((unsigned)__double2hiint(c));
    if (e - 898u > 249u || eb - 898u > 249u || ed - 898u > 249u || ea - 127u > 1792u || ec - 127u > 1792u) {
        q1 = div_nr(a, b);
        q2 = div_nr(c, d);
        return;
    }
    const double r = rcp_refine(bd, (unsigned)__double2hiint(bd), e);
    q1 = __dmul_rn(a, __dmul_rn(d, r));
    q2 = __dmul_rn(c, __dmul_rn(b, r));
}

// The face sweep's forms in the arithmetic type T: binary32 keeps the hardware operations.
template <typename T> __device__ __forceinline__ T sw_rcp(T y) { return T(1) / y; }
template <typename T> __device__ __forceinline__ T sw_div(T x, T y) { return x / y; }
template <typename T> __device__ __forceinline__ T sw_sqrt(T x) { return sqrtf(x); }
template <> __device__ __forceinline__ double sw_rcp(double y) { return rcp_nr(y); }
template <> __device__ __forceinline__ double sw_div(double x, double y) { return div_nr(x, y); }
template <> __device__ __forceinline__ double sw_sqrt(double x) { return sqrt_nr(x); }
template <typename T> __device__ __forceinline__ void sw_div2(T a, T b, T c, T d, T &q1, T &q2)
{
    q1 = a / b;
    q2 = c / d;
}
template <> __device__ __forceinline__ void sw_div2(double a, double b, double c, double d, double &q1, double &q2)
{
    div2_nr(a, b, c, d, q1, q2);
}

// The reference's wp.min / wp.max / wp.sign: a < b ? a : b, a > b ? a : b, x < 0 ? -1 : 1
// (binary64: by the integer compares above, the same results).
template <typename T> __device__ __forceinline__ T wmin(T a, T b) { return a < b ? a : b; }
template <typename T> __device__ __forceinline__ T wmax(T a, T b) { return a > b ? a : b; }
template <typename T> __device__ __forceinline__ T wsign(T x) { return x < T(0) ? T(-1) : T(1); }
template <> __device__ __forceinline__ double wmin(double a, double b) { return dlt(a, b) ? a : b; }
template <> __device__ __forceinline__ double wmax(double a, double b) { return dlt(b, a) ? a : b; }
template <> __device__ __forceinline__ double wsign(double x) { return dneg(x) ? -1.0 : 1.0; }
__device__ __forceinline__ double wabs(double x) { return fabs(x); }
__device__ __forceinline__ float wabs(float x) { return fabsf(x); }
__device__ __forceinline__ bool wisnan(double x)  // by integer compare of the bits, in PTX as dlt
{
    unsigned r;
    asm("{\n\t.reg .s64 m;\n\t.reg .pred p;\n\tmov.b64 m, %1;\n\t"
        "and.b64 m, m, 0x7fffffffffffffff;\n\tsetp.gt.s64 p, m, 0x7ff0000000000000;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r) : "d"(x));
    return r != 0u;
}
__device__ __forceinline__ bool wisnan(float x) { return isnan(x); }
__device__ __forceinline__ double wfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float wfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double wsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float wsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double wtanh(double x) { return tanh(x); }
__device__ __forceinline__ float wtanh(float x) { return tanhf(x); }
__device__ __forceinline__ double wpow(double a, double b) { return pow(a, b); }
__device__ __forceinline__ float wpow(float a, float b) { return powf(a, b); }

template <typename T> struct S6 { T v[6]; };

// ------------------------------------------------------------------------------------------------
// Mixture stiffened-gas EOS (SC:83-110)
// ------------------------------------------------------------------------------------------------
// Gamma = sum a_k/(g_k-1), Pi = sum a_k g_k pi_k/(g_k-1), with a2 = 1 - a1: linear in a1, so each
// is one fused multiply-add from the second fluid's value and the slope (r1 - r2, k1 - k2, formed
// once on the host) -- within a unit or two in the last place of the two-product sum.
template <typename T>
__device__ __forceinline__ void mix_gamma_pibig(const Eos &e, T a1, T &gb, T &pb)
{
    gb = wfma(a1, cst<T>(e.dr, e.drf), cst<T>(e.r2, e.r2f));
    pb = wfma(a1, cst<T>(e.dk, e.dkf), cst<T>(e.k2, e.k2f));
}

// mixture gamma and p_inf: g = 1/Gamma + 1, p_inf = (g-1) Pi / g = Pi / (1 + Gamma), with the two
// reciprocals taken from one division 1 / (Gamma (1 + Gamma)). SW: the face sweep's reciprocal.
// mix_from_pibig: the same from Gamma and Pi already at hand; mix_from_gp1 with gp1 = 1 + Gamma too.
template <typename T, bool SW = false>
__device__ __forceinline__ void mix_from_gp1(T gb, T gp1, T pb, T &g, T &pi)
{
    const T inv = SW ? sw_rcp(gb * gp1) : T(1) / (gb * gp1);
    g = gp1 * inv + T(1);
    pi = pb * (gb * inv);
}
template <typename T, bool SW = false>
__device__ __forceinline__ void mix_from_pibig(T gb, T pb, T &g, T &pi)
{
    mix_from_gp1<T, SW>(gb, T(1) + gb, pb, g, pi);
}
template <typename T, bool SW = false>
__device__ __forceinline__ void mix_gamma_pinf(const Eos &e, T a1, T &g, T &pi)
{
    T gb, pb;
    mix_gamma_pibig(e, a1, gb, pb);
    mix_from_pibig<T, SW>(gb, pb, g, pi);
}

// sound_speed(rho, p, a1) with 1/rho supplied. SW (the face sweep): the square root and, in
// binary64, c^2 = g (p + p_inf) / rho written with the mixture's Gamma and Pi as
// ((1 + Gamma) p + Pi) / (Gamma rho) (g = 1 + 1/Gamma, p_inf = Pi / (1 + Gamma)): one reciprocal
// instead of mix_gamma_pinf's, the same value up to rounding.
template <typename T, bool SW = false>
__device__ __forceinline__ T sound_speed_r(const Eos &e, T inv_rho, T p, T a1)
{
    T val;
    if constexpr (SW && sizeof(T) == 8) {
        T gb, pb;
        mix_gamma_pibig(e, a1, gb, pb);
        val = ((T(1) + gb) * p + pb) * inv_rho * sw_rcp(gb);
    } else {
        T g, pi;
        mix_gamma_pinf<T, SW>(e, a1, g, pi);
        val = g * (p + pi) * inv_rho;
    }
    if (flt(val, T(kTiny))) val = T(kTiny);
    return SW ? sw_sqrt(val) : wsqrt(val);
}

// prim_to_energy (SC:105-110)
template <typename T>
__device__ __forceinline__ T prim_to_energy(const Eos &e, T rho, T u, T v, T p, T a1)
{
    T gb, pb;
    mix_gamma_pibig(e, a1, gb, pb);
    return gb * p + pb + T(0.5) * rho * (u * u + v * v);
}

// ------------------------------------------------------------------------------------------------
// Positivity helpers (SC:112-292)
// ------------------------------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T clamp01_pp(T a1)
{
    T a = a1;
    if (wisnan(a)) a = T(kPpAlpha);
    if (flt(a, T(kPpAlpha))) a = T(kPpAlpha);
    if (fgt(a, T(1) - T(kPpAlpha))) a = T(1) - T(kPpAlpha);
    return a;
}

// True when clamp01_pp leaves a binary64 a1 unchanged: a1 in [kPpAlpha, 1 - kPpAlpha]. Positive
// binary64 values order like their bit patterns, and negative values, NaN and values outside map
// above the range after the unsigned subtraction, so one unsigned compare of the bits decides --
// on the integer pipe (clamp01_pp's compares and selects were measured at three binary64-pipe
// instructions).
__device__ __forceinline__ bool alpha_inside(double a1)
{
    constexpr unsigned long long lo = 0x3DDB7CDFD9D7BDBBull;  // bits of kPpAlpha = 1e-10
    constexpr unsigned long long hi = 0x3FEFFFFFFFF24190ull;  // bits of 1 - kPpAlpha
    return (unsigned long long)__double_as_longlong(a1) - lo <= hi - lo;
}

__device__ __forceinline__ double pp_theta_lower(double base, double high, double floor_)
{
    double theta = 1.0;
    if (isnan(base) || isnan(high)) {
        theta = 0.0;
    } else if (high < floor_) {
        double denom = base - high;
        theta = denom > kTiny ? (base - floor_) / denom : 0.0;
    }
    if (theta < 0.0) theta = 0.0;
    if (theta > 1.0) theta = 1.0;
    return theta;
}

template <typename T>
__device__ __forceinline__ S6<T> blend_s6(const S6<T> &base, const S6<T> &high, T theta)
{
    S6<T> s;
#pragma unroll
    for (int f = 0; f < 6; ++f) s.v[f] = base.v[f] + theta * (high.v[f] - base.v[f]);
    return s;
}

// rho c~^2 of an SC state [m1, m2, rho u, rho v, p, alpha] (SC:174-178)
template <typename T> __device__ __forceinline__ T rho_ctilde2_sc(const Eos &e, const S6<T> &s)
{
    T g, pi;
    mix_gamma_pinf(e, clamp01_pp(s.v[5]), g, pi);
    return (s.v[4] + pi) / (g - T(1));
}

template <typename T> __device__ __forceinline__ S6<T> pp_floor_pressure_state(const Eos &e, S6<T> s)
{
    T a1 = clamp01_pp(s.v[5]);
    T g, pi;
    mix_gamma_pinf(e, a1, g, pi);
    if (wisnan(s.v[4]) || flt(rho_ctilde2_sc(e, s), T(kPpCtilde))) s.v[4] = T(kPpCtilde) * (g - T(1)) - pi;
    s.v[5] = a1;
    return s;
}

template <typename T>
__device__ __forceinline__ S6<T> wong_stage_lower_s6(const S6<T> &base, const S6<T> &high, T base_val,
                                                     T high_val, T floor_)
{
    T theta = T(1);
    if (wisnan(base_val) || wisnan(high_val) || flt(base_val, floor_)) {
        theta = T(0);
    } else if (flt(high_val, floor_)) {
        T denom = base_val - high_val;
        theta = fgt(denom, T(kTiny)) ? (base_val - floor_) / denom : T(0);
    }
    return blend_s6(base, high, theta);
}

// Wong staged interpolation limiter on a reconstructed state (SC:217-240, used by M10:1007-1008)
template <typename T>
__device__ __forceinline__ S6<T> pp_limit_reconstructed_state(const Eos &e, const S6<T> &high,
                                                              const S6<T> &base)
{
    S6<T> b = base;
    b.v[5] = clamp01_pp(b.v[5]);
    if (flt(b.v[0], T(kPpRho)) || wisnan(b.v[0])) b.v[0] = T(kPpRho);
    if (flt(b.v[1], T(kPpRho)) || wisnan(b.v[1])) b.v[1] = T(kPpRho);
    S6<T> s = high;
    s = wong_stage_lower_s6(b, s, b.v[0], s.v[0], T(kPpRho));
    s = wong_stage_lower_s6(b, s, b.v[1], s.v[1], T(kPpRho));
    s = wong_stage_lower_s6(b, s, b.v[5], s.v[5], T(kPpAlpha));
    s = wong_stage_lower_s6(b, s, T(1) - b.v[5], T(1) - s.v[5], T(kPpAlpha));
    s = wong_stage_lower_s6(b, s, rho_ctilde2_sc(e, b), rho_ctilde2_sc(e, s), T(kPpCtilde));
    if (flt(s.v[0], T(kPpHsRho)) || flt(s.v[1], T(kPpHsRho)) || flt(s.v[5], T(kPpHsAlpha)) ||
        fgt(s.v[5], T(1) - T(kPpHsAlpha)))
        s = b;
    if (flt(rho_ctilde2_sc(e, s), T(kPpHsCtilde)) || wisnan(s.v[4])) s = b;
    return s;
}

// rho c~^2 = E - kinetic - pi of a conserved state (SC:242-258); always binary64.
__device__ __forceinline__ double rho_ctilde2_cons(const Eos &e, double m1, double m2, double mx,
                                                   double my, double E, double a1_in)
{
    double a1 = clamp01_pp(a1_in);
    double mm1 = m1, mm2 = m2;
    if (mm1 < kPpRho || isnan(mm1)) mm1 = kPpRho;
    if (mm2 < kPpRho || isnan(mm2)) mm2 = kPpRho;
    double rho = mm1 + mm2;
    double ir = 1.0 / rho;
    double uu = mx * ir, vv = my * ir;
    double kin = 0.5 * rho * (uu * uu + vv * vv);
    double g, pi;
    mix_gamma_pinf(e, a1, g, pi);
    return E - kin - pi;
}

// Limiter factor of pass 2 (the rho c~^2 bound of theta_cons_stage, SC:283-286) evaluating the
// low-order bound value only when it can change the result: pp_theta_lower returns 1 when the
// high-order value is at or above the floor and neither value is NaN, and the low-order value
// lc = E - kin - p_inf can only be NaN when one of l[2..4] is not finite.
// True when rho c~^2 = E - kin - p_inf of the conserved state (m1, m2, mx, my, E, a1_in) is
// certainly >= `floor_`, decided without a division: with rho > 0 and 1 + Gamma > 0,
//   E - (mx^2 + my^2) / (2 rho) - Pi / (1 + Gamma) >= floor
//   <=>  2 rho (1 + Gamma) (E - floor) - (1 + Gamma) (mx^2 + my^2) - 2 rho Pi >= 0,
// and a margin of 1e-12 of the terms' magnitude keeps every case that round-off could decide
// either way for the exact formula (rho_ctilde2_cons).
__device__ __forceinline__ bool ctilde_surely_above(const Eos &e, double m1, double m2, double mx,
                                                    double my, double E, double a1_in, double floor_)
{
    double a1 = clamp01_pp(a1_in);
    double mm1 = m1, mm2 = m2;
    if (mm1 < kPpRho || isnan(mm1)) mm1 = kPpRho;
    if (mm2 < kPpRho || isnan(mm2)) mm2 = kPpRho;
    double rho = mm1 + mm2;
    double gb, pb;
    mix_gamma_pibig(e, a1, gb, pb);
    double gp1 = 1.0 + gb;
    double t1 = 2.0 * rho * gp1 * (E - floor_);
    double t2 = gp1 * (mx * mx + my * my);
    double t3 = 2.0 * rho * pb;
    double sgn = t1 - t2 - t3;
    return sgn > 1e-12 * (fabs(t1) + t2 + fabs(t3));  // false for NaN
}

__device__ __forceinline__ double theta_ctilde(const Eos &e, const double l[6], const double h[6])
{
    double theta;
    if (ctilde_surely_above(e, h[0], h[1], h[2], h[3], h[4], h[5], kPpCtilde) && isfinite(l[2]) &&
        isfinite(l[3]) && isfinite(l[4])) {
        theta = 1.0;
    } else {
        double hc = rho_ctilde2_cons(e, h[0], h[1], h[2], h[3], h[4], h[5]);
        double lc = rho_ctilde2_cons(e, l[0], l[1], l[2], l[3], l[4], l[5]);
        theta = pp_theta_lower(lc, hc, kPpCtilde);
    }
    if (theta < 0.0 || isnan(theta)) theta = 0.0;
    if (theta > 1.0) theta = 1.0;
    return theta;
}

// Limiter factor of one cell for one pass (theta_cons_stage, SC:268-292); binary64.
__device__ __forceinline__ double theta_cons_stage(const Eos &e, const double l[6], const double h[6],
                                                   int stage)
{
    double theta = 1.0;
    if (stage == 0) {
        theta = wmin(theta, pp_theta_lower(l[0], h[0], kPpRho));
        theta = wmin(theta, pp_theta_lower(l[1], h[1], kPpRho));
    } else if (stage == 1) {
        theta = wmin(theta, pp_theta_lower(l[5], h[5], kPpAlpha));
        theta = wmin(theta, pp_theta_lower(1.0 - l[5], 1.0 - h[5], kPpAlpha));
    } else {
        double lc = rho_ctilde2_cons(e, l[0], l[1], l[2], l[3], l[4], l[5]);
        double hc = rho_ctilde2_cons(e, h[0], h[1], h[2], h[3], h[4], h[5]);
        theta = pp_theta_lower(lc, hc, kPpCtilde);
    }
    if (theta < 0.0 || isnan(theta)) theta = 0.0;
    if (theta > 1.0) theta = 1.0;
    return theta;
}

// ------------------------------------------------------------------------------------------------
// Limiters and sensors (SC:295-325)
// ------------------------------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T mm2(T x, T y)
{
    return T(0.5) * (wsign(x) + wsign(y)) * wmin(wabs(x), wabs(y));
}

template <typename T> __device__ __forceinline__ T mm4(T a, T b, T c, T d)
{
    T sa = wsign(a);
    T s = sa + wsign(b);
    return T(0.125) * s * wabs((sa + wsign(c)) * (sa + wsign(d))) *
           wmin(wmin(wabs(a), wabs(b)), wmin(wabs(c), wabs(d)));
}

// |x| < c for c > 0 (false for NaN x): binary64 by the magnitude's bit pattern in PTX (a fabs
// feeding the integer compare would be formed by a binary64 addition).
template <typename T> __device__ __forceinline__ bool abs_lt(T x, T c) { return flt(wabs(x), c); }
template <> __device__ __forceinline__ bool abs_lt(double x, double c)
{
    unsigned r;
    asm("{\n\t.reg .s64 m, k;\n\t.reg .pred p;\n\tmov.b64 m, %1;\n\tmov.b64 k, %2;\n\t"
        "and.b64 m, m, 0x7fffffffffffffff;\n\tsetp.lt.s64 p, m, k;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r) : "d"(x), "d"(c));
    return r != 0u;
}

// Binary64 mm2 / mm4 on the integer pipe, the same values as the products above: with the signs
// of wsign (x < 0 ? -1 : 1) and m the a<b?a:b minimum of the magnitudes, the sign sum and product
// are +-2 / +-4 when the signs agree (the result is +-m, negated by its sign bit) and 0 otherwise
// (the result is 0 times m: a zero -- negative for mm4 when a and b are negative, the sign of
// 0.125 s -- or NaN when m is infinite or NaN).
__device__ __forceinline__ double with_sign(double m, bool neg)
{
    return __longlong_as_double(__double_as_longlong(m) ^ (neg ? (long long)0x8000000000000000ULL : 0LL));
}
__device__ __forceinline__ double zero_times(double m, bool neg)
{
    const bool finite = (__double_as_longlong(m) & 0x7fffffffffffffffLL) < 0x7ff0000000000000LL;
    return finite ? with_sign(0.0, neg) : __longlong_as_double(0x7ff8000000000000LL);
}
// wmin(|x|, |y|) on the magnitudes' bit patterns (in PTX: a fabs feeding an integer compare would
// be formed by a binary64 operation): |x| when |x| < |y| with neither NaN, else |y|.
__device__ __forceinline__ double min_mag(double x, double y)
{
    double r;
    asm("{\n\t.reg .s64 mx, my;\n\t.reg .pred p;\n\tmov.b64 mx, %1;\n\tmov.b64 my, %2;\n\t"
        "and.b64 mx, mx, 0x7fffffffffffffff;\n\tand.b64 my, my, 0x7fffffffffffffff;\n\t"
        "setp.le.s64 p, mx, 0x7ff0000000000000;\n\tsetp.le.and.s64 p, my, 0x7ff0000000000000, p;\n\t"
        "setp.lt.and.s64 p, mx, my, p;\n\tselp.b64 mx, mx, my, p;\n\tmov.b64 %0, mx;\n\t}"
        : "=d"(r) : "d"(x), "d"(y));
    return r;
}
template <> __device__ __forceinline__ double mm2(double x, double y)
{
    const double m = min_mag(x, y);
    const bool nx = dneg(x);
    return nx == dneg(y) ? with_sign(m, nx) : zero_times(m, false);
}
template <> __device__ __forceinline__ double mm4(double a, double b, double c, double d)
{
    // wmin(wmin(|a|, |b|), wmin(|c|, |d|)): the inner minima are magnitudes (or NaN), so the outer
    // one is min_mag of them
    const double m = min_mag(min_mag(a, b), min_mag(c, d));
    const bool na = dneg(a), nb = dneg(b);
    if (na == nb && na == dneg(c) && na == dneg(d)) return with_sign(m, na);
    return zero_times(m, na && nb);
}

// x / 2: binary64 by subtracting 1 from the exponent on the integer pipe (the exact product) where
// the result stays normal; zeros, subnormals, the smallest normals, infinities and NaN multiply.
// x * c for the rare operands of the exponent-arithmetic forms below, out of line: inline, the
// compiler evaluated the product for every operand (measured: one binary64 multiply per call).
static __device__ __noinline__ double scaled_rare(double x, double c) { return x * c; }

template <typename T> __device__ __forceinline__ T half_of(T x) { return T(0.5) * x; }
template <> __device__ __forceinline__ double half_of(double x)
{
    const long long b = __double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    return e - 2u < 2045u ? __longlong_as_double(b - (1LL << 52)) : scaled_rare(x, 0.5);
}

// 0.5 (1 + s) a + 0.5 (1 - s) b for s = wsign(.) = +-1 (the interface velocity of hllc_x_src,
// SC:760-768): one coefficient is 1 and the other 0, so the value is the chosen term plus 0 times
// the other (a zero of the other's sign, or NaN when it is infinite or NaN). Binary64: that sum
// on the integer pipe and one addition; binary32: the products.
template <typename T> __device__ __forceinline__ T sign_select(T s, T a, T b)
{
    return T(0.5) * (T(1) + s) * a + T(0.5) * (T(1) - s) * b;
}
template <> __device__ __forceinline__ double sign_select(double s, double a, double b)
{
    const bool pick_a = !dneg(s);
    const double other = pick_a ? b : a;  // (+0) other: a zero with other's sign bit, or NaN
    return (pick_a ? a : b) + zero_times(other, __double_as_longlong(other) < 0);
}

// p / rho^gamma(alpha) (SC:308-314)
template <typename T> __device__ __forceinline__ T cell_entropy(const Eos &e, T ar1, T ar2, T p, T a1)
{
    T rho = ar1 + ar2;
    if (rho < T(kTiny)) rho = T(kTiny);
    T g, pi;
    mix_gamma_pinf(e, a1, g, pi);
    return p / wpow(rho, g);
}

// smoothness indicator (SC:318-325)
template <typename T> __device__ __forceinline__ T cator2_val(T em2, T em1, T e0, T ep1, T ep2)
{
    T aa = T(0.25) * wabs(em2 - T(4) * em1 + T(3) * e0) + T(13.0 / 12.0) * wabs(e0 - T(2) * em1 + em2);
    T bb = T(0.25) * wabs(T(3) * e0 - T(4) * ep1 + ep2) + T(13.0 / 12.0) * wabs(e0 - T(2) * ep1 + ep2);
    return (T(2) * aa * bb + T(kYuxin)) / (aa * aa + bb * bb + T(kYuxin));
}

// ------------------------------------------------------------------------------------------------
// Reconstructions (SC:327-446)
// ------------------------------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T thinc_ul(const Eos &e, T vm1, T v0, T v1)
{
    T result = v0;
    if (fpos((v1 - v0) * (v0 - vm1))) {
        T qa = T(0.5) * (v1 + vm1);
        T qd = T(0.5) * (v1 - vm1);
        T feng = sw_div(v0 - qa, qd);
        T T1 = cst<T>(e.thinc_t1, e.thinc_t1f);
        T T2 = wtanh(feng * T(1.8) * T(0.5));
        result = qa + sw_div(qd * (T1 + T2 * cst<T>(e.thinc_inv_t1, e.thinc_inv_t1f)), T(1) + T2);
    }
    return result;
}

template <typename T> __device__ __forceinline__ T thinc_ur(const Eos &e, T v0, T v1, T v2)
{
    T result = v1;
    if (fpos((v2 - v1) * (v1 - v0))) {
        T qa = T(0.5) * (v2 + v0);
        T qd = T(0.5) * (v2 - v0);
        T feng = sw_div(v1 - qa, qd);
        T T1 = cst<T>(e.thinc_t1, e.thinc_t1f);
        T T2 = wtanh(feng * T(1.8) * T(0.5));
        result = qa - sw_div(qd * (T1 - T2 * cst<T>(e.thinc_inv_t1, e.thinc_inv_t1f)), T(1) - T2);
    }
    return result;
}

// MP5's alpha x slope, alpha = 4: binary64 by adding 2 to the exponent on the integer pipe (the
// exact product) where the result stays normal and finite; zeros, subnormals, infinities and NaN,
// and values whose product would overflow, take the multiplication.
static_assert(kMp5Alpha == 4.0, "mp5_alpha_times assumes alpha = 4");
template <typename T> __device__ __forceinline__ T mp5_alpha_times(T x)
{
    if constexpr (sizeof(T) == 8) {
        const long long b = __double_as_longlong(x);
        const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
        return e - 1u < 2044u ? __longlong_as_double(b + (2LL << 52)) : scaled_rare(x, 4.0);
    } else {
        return T(kMp5Alpha) * x;
    }
}

// Suresh-Huynh MP5, left-biased value at i+1/2 from cells i-2..i+2 (SC:353-377). The binary32
// sweep's form; the binary64 sweep uses mp5_diff.
template <typename T> __device__ __forceinline__ T mp5_ul(T vm2, T vm1, T v0, T vp1, T vp2)
{
    T VOR = T(k1o60) * (T(2) * vm2 - T(13) * vm1 + T(47) * v0 + T(27) * vp1 - T(3) * vp2);
    T VMP = v0 + mm2(vp1 - v0, mp5_alpha_times(v0 - vm1));
    T result = VOR;
    if (fge((VOR - v0) * (VOR - VMP), T(kEpsM))) {
        T DJM1 = vm2 - T(2) * vm1 + v0;
        T DJ = vm1 - T(2) * v0 + vp1;
        T DJP1 = v0 - T(2) * vp1 + vp2;
        T DM4JPH = mm4(T(4) * DJ - DJP1, T(4) * DJP1 - DJ, DJ, DJP1);
        T DM4JMH = mm4(T(4) * DJ - DJM1, T(4) * DJM1 - DJ, DJ, DJM1);
        T VUL = v0 + T(kMp5Alpha) * (v0 - vm1);
        T VAV = T(0.5) * (v0 + vp1);
        T VMD = VAV - T(0.5) * DM4JPH;
        T VLC = v0 + T(0.5) * (v0 - vm1) + T(kB2) * DM4JMH;
        T VMIN = wmax(wmin(wmin(v0, vp1), VMD), wmin(wmin(v0, VUL), VLC));
        T VMAX = wmin(wmax(wmax(v0, vp1), VMD), wmax(wmax(v0, VUL), VLC));
        result = VOR + mm2(VMIN - VOR, VMAX - VOR);
    }
    return result;
}

// MP5 in difference form (binary64 sweep): the value at the face from the stencil's centre c, the
// neighbour across the face p1 = v(+1), and the differences dm2 = v(-1) - v(-2), dm1 = c - v(-1),
// d0 = p1 - c, d1 = v(+2) - p1 -- the left-biased value of mp5_ul with (vm2, vm1, v0, vp1, vp2).
// The same terms, each from differences:
// VOR - v0 = (-2 dm2 + 11 dm1 + 24 d0 - 3 d1) / 60 (the five-point weights sum to 1), the test
// (VOR - v0)(VOR - VMP) >= eps with VMP - v0 = mm2(d0, 4 dm1), the second differences
// DJM1 = dm1 - dm2, DJ = d0 - dm1, DJP1 = d1 - d0, VUL = v0 + 4 dm1, VAV = v0 + d0 / 2,
// VLC = v0 + dm1 / 2 + 4/3 DM4JMH. The right-biased value of mp5_ur at the same face is this
// function of the mirrored stencil: centre vp1, neighbour v0 and differences -(vp3 - vp2),
// -(vp2 - vp1), -(vp1 - v0), -(v0 - vm1) (every term of mp5_ur maps onto one of mp5_ul). One subtraction per
// difference, shared by the two values of a field, replaces the stencil sums; values equal the
// reference's up to rounding.
__device__ __forceinline__ double mp5_diff(double c, double p1, double dm2, double dm1, double d0, double d1)
{
    const double D = (-2.0 / 60.0) * dm2 + (11.0 / 60.0) * dm1 + (24.0 / 60.0) * d0 - (3.0 / 60.0) * d1;
    const double VOR = c + D;
    const double m = mm2(d0, mp5_alpha_times(dm1));
    // The test D (D - m) >= eps cannot pass when D is +-0, or when D and m have the same sign bit
    // and |m| > |D|: D - m is then nonzero with D's opposite sign, so the product is negative (a NaN
    // or infinite m makes it NaN or negative). Settled on the integer pipe from the bits -- the
    // same decision -- it skips the binary64 difference and product for nearly every smooth or
    // flat stencil.
    const long long bD = __double_as_longlong(D), bm = __double_as_longlong(m);
    const long long aD = bD & 0x7fffffffffffffffLL, am = bm & 0x7fffffffffffffffLL;
    if (aD == 0 || ((bD ^ bm) >= 0 && am > aD)) return VOR;
    if (!fge(D * (D - m), kEpsM)) return VOR;
    const double DJM1 = dm1 - dm2, DJ = d0 - dm1, DJP1 = d1 - d0;
    const double DM4JPH = mm4(4.0 * DJ - DJP1, 4.0 * DJP1 - DJ, DJ, DJP1);
    const double DM4JMH = mm4(4.0 * DJ - DJM1, 4.0 * DJM1 - DJ, DJ, DJM1);
    const double VUL = c + mp5_alpha_times(dm1);
    const double VAV = c + half_of(d0);
    const double VMD = VAV - 0.5 * DM4JPH;
    const double VLC = c + half_of(dm1) + kB2 * DM4JMH;
    const double VMIN = wmax(wmin(wmin(c, p1), VMD), wmin(wmin(c, VUL), VLC));
    const double VMAX = wmin(wmax(wmax(c, p1), VMD), wmax(wmax(c, VUL), VLC));
    return VOR + mm2(VMIN - VOR, VMAX - VOR);
}

// right-biased value at i+1/2 from cells i-1..i+3 (SC:379-405)
template <typename T> __device__ __forceinline__ T mp5_ur(T vm1, T v0, T vp1, T vp2, T vp3)
{
    T VOR = T(k1o60) * (T(-3) * vm1 + T(27) * v0 + T(47) * vp1 - T(13) * vp2 + T(2) * vp3);
    T VMP = vp1 + mm2(v0 - vp1, mp5_alpha_times(vp1 - vp2));
    T result = VOR;
    if (fge((VOR - vp1) * (VOR - VMP), T(kEpsM))) {
        T DJM1 = vm1 - T(2) * v0 + vp1;
        T DJ = v0 - T(2) * vp1 + vp2;
        T DJP1 = vp1 - T(2) * vp2 + vp3;
        T DM4JPH = mm4(T(4) * DJ - DJP1, T(4) * DJP1 - DJ, DJ, DJP1);
        T DM4JMH = mm4(T(4) * DJ - DJM1, T(4) * DJM1 - DJ, DJ, DJM1);
        T VUL = vp1 + T(kMp5Alpha) * (vp1 - vp2);
        T VAV = T(0.5) * (vp1 + v0);
        T VMD = VAV - T(0.5) * DM4JMH;
        T VLC = vp1 + T(0.5) * (vp1 - vp2) + T(kB2) * DM4JPH;
        T VMIN = wmax(wmin(wmin(vp1, v0), VMD), wmin(wmin(vp1, VUL), VLC));
        T VMAX = wmin(wmax(wmax(vp1, v0), VMD), wmax(wmax(vp1, VUL), VLC));
        result = VOR + mm2(VMIN - VOR, VMAX - VOR);
    }
    return result;
}

// sixth-order central face value (SC:407-412)
// binary64: the mean of the two five-point values as one six-point combination,
// (2 vm2 - 16 vm1 + 74 v0 + 74 vp1 - 16 vp2 + 2 vp3) / 120.
template <typename T> __device__ __forceinline__ T central6_avg(T vm2, T vm1, T v0, T vp1, T vp2, T vp3)
{
    if constexpr (sizeof(T) == 8) {
        return (1.0 / 60.0) * (vm2 + vp3) - (8.0 / 60.0) * (vm1 + vp2) + (37.0 / 60.0) * (v0 + vp1);
    } else {
        T left = T(k1o60) * (T(2) * vm2 - T(13) * vm1 + T(47) * v0 + T(27) * vp1 - T(3) * vp2);
        T right = T(k1o60) * (T(-3) * vm1 + T(27) * v0 + T(47) * vp1 - T(13) * vp2 + T(2) * vp3);
        return T(0.5) * (left + right);
    }
}

// fourth-order central face value (SC:1076-1082)
template <typename T> __device__ __forceinline__ T central4(T wm1, T w0, T w1, T w2)
{
    return -T(1.0 / 12.0) * wm1 + T(7.0 / 12.0) * w0 + T(7.0 / 12.0) * w1 - T(1.0 / 12.0) * w2;
}

// MUSCL kappa=1/3 on a characteristic field (SC:430-446)
template <typename T> __device__ __forceinline__ T muscl_char_ul(T vm1, T v0, T vp1)
{
    T dm = v0 - vm1;
    T d0 = vp1 - v0;
    return v0 + T(0.25) * (T(1.0 - kKappa) * mm2(dm, T(2) * d0) + T(1.0 + kKappa) * mm2(d0, T(2) * dm));
}

template <typename T> __device__ __forceinline__ T muscl_char_ur(T v0, T vp1, T vp2)
{
    T dp = vp2 - vp1;
    T d0 = vp1 - v0;
    return vp1 - T(0.25) * (T(1.0 - kKappa) * mm2(dp, T(2) * d0) + T(1.0 + kKappa) * mm2(d0, T(2) * dp));
}

// ------------------------------------------------------------------------------------------------
// Characteristic projections with face-averaged eigenvectors (SC:447-589).
// State order [ar1, ar2, rho u, rho v, p, alpha1]; DIR 0 = x faces, 1 = y faces.
// ------------------------------------------------------------------------------------------------
template <typename T> struct FaceBasis {
    T c, c2, inv2c, inv2c2, Y1, Y2, Y1c2, Y2c2, u, v;
};

template <int DIR, typename T> __device__ __forceinline__ S6<T> to_char(const FaceBasis<T> &b, const T u[6])
{
    S6<T> s;
    if constexpr (sizeof(T) == 4) {  // binary32: the rows as the reference writes them
        if (DIR == 0) {  // to_char_x (SC:480-499)
            T un = b.u, ut = b.v;
            s.v[0] = un * b.inv2c * u[0] + un * b.inv2c * u[1] - b.inv2c * u[2] + b.inv2c2 * u[4];
            s.v[1] = u[0] - b.Y1c2 * u[4];
            s.v[2] = u[1] - b.Y2c2 * u[4];
            s.v[3] = -ut * u[0] - ut * u[1] + u[3];
            s.v[4] = u[5];
            s.v[5] = -un * b.inv2c * u[0] - un * b.inv2c * u[1] + b.inv2c * u[2] + b.inv2c2 * u[4];
        } else {  // to_char_y (SC:537-556)
            T un = b.v, ut_f = -b.u;
            s.v[0] = un * b.inv2c * u[0] + un * b.inv2c * u[1] - b.inv2c * u[3] + b.inv2c2 * u[4];
            s.v[1] = u[0] - b.Y1c2 * u[4];
            s.v[2] = u[1] - b.Y2c2 * u[4];
            s.v[3] = -ut_f * u[0] - ut_f * u[1] - u[2];
            s.v[4] = u[5];
            s.v[5] = -un * b.inv2c * u[0] - un * b.inv2c * u[1] + b.inv2c * u[3] + b.inv2c2 * u[4];
        }
        return s;
    }
    // Binary64: the same rows with the partial densities' sum and the acoustic rows' common part
    // formed once: w0 = A + C and w5 = C - A for A = (un (u0 + u1) - m_n) / (2c), C = p / (2c^2),
    // un the normal velocity, m_n the normal momentum.
    constexpr int N = DIR == 0 ? 2 : 3;  // normal momentum field
    const T un = DIR == 0 ? b.u : b.v;
    const T s01 = u[0] + u[1];
    const T A = un * b.inv2c * s01 - b.inv2c * u[N];
    const T C = b.inv2c2 * u[4];
    s.v[0] = A + C;
    s.v[1] = u[0] - b.Y1c2 * u[4];
    s.v[2] = u[1] - b.Y2c2 * u[4];
    if (DIR == 0)  // to_char_x (SC:480-499): -v (u0 + u1) + u3
        s.v[3] = u[3] - b.v * s01;
    else  // to_char_y (SC:537-556): u (u0 + u1) - u2
        s.v[3] = -(u[2] - b.u * s01);
    s.v[4] = u[5];
    s.v[5] = C - A;
    return s;
}

template <int DIR, typename T> __device__ __forceinline__ S6<T> to_phys(const FaceBasis<T> &b, const T w[6])
{
    S6<T> s;
    s.v[0] = b.Y1 * (w[0] + w[5]) + w[1];
    s.v[1] = b.Y2 * (w[0] + w[5]) + w[2];
    if (DIR == 0) {  // to_phys_x (SC:504-534)
        s.v[2] = (b.u - b.c) * w[0] + b.u * w[1] + b.u * w[2] + (b.u + b.c) * w[5];
        s.v[3] = b.v * (w[0] + w[1] + w[2] + w[5]) + w[3];
    } else {  // to_phys_y (SC:559-589)
        s.v[2] = b.u * (w[0] + w[1] + w[2] + w[5]) - w[3];
        s.v[3] = (b.v - b.c) * w[0] + b.v * w[1] + b.v * w[2] + (b.v + b.c) * w[5];
    }
    s.v[4] = b.c2 * (w[0] + w[5]);
    s.v[5] = w[4];
    return s;
}

// ------------------------------------------------------------------------------------------------
// HLLC flux and interface velocity (SC:594-771). One side's state with its sound speed and energy.
// ------------------------------------------------------------------------------------------------
template <typename T> struct Side {
    T ar1, ar2, rho, un, ut, p, a, c, E;
    T gb, pb;  // the mixture's Gamma and Pi (hllc with LAZY_E forms E from them)
};

// Flux f[0..5] in SC component order and the interface velocity u* for the alpha source.
// hllc_x/hllc_y and hllc_x_src/hllc_y_src of the reference recompute the same wave speeds; here
// they are computed once.
// LAZY_E: the sides carry Gamma and Pi instead of E, and hllc forms the total energy of the one side
// its branch reads (L for the left and star-left fluxes, R for the others) by prim_to_energy's
// expression -- the same value, for one side instead of two.
// The wave speeds S_L, S_R and the contact speed S_P of hllc, the first part of it (shared, so that
// a caller that needs only these gets hllc's own values).
template <typename T>
__device__ __forceinline__ void hllc_speeds(const Side<T> &L, const Side<T> &R, T &SL, T &SR, T &SP)
{
    T n_avg = half_of(L.un + R.un);
    T c_avg = half_of(L.c + R.c);
    SL = wmin(L.un - L.c, n_avg - c_avg);
    SR = wmax(R.un + R.c, n_avg + c_avg);
    T denom = L.rho * (SL - L.un) - R.rho * (SR - R.un);
    if (abs_lt(denom, T(kTiny))) denom = T(kTiny);
    SP = sw_div(R.p - L.p + L.rho * L.un * (SL - L.un) - R.rho * R.un * (SR - R.un), denom);
}

// |x| <= 2^60 and finite, |x| >= 2^-60: integer tests of a binary64's magnitude bits.
__device__ __forceinline__ bool mag_at_most_2p60(double x)
{
    return ((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull) <= 0x43B0000000000000ull;
}
__device__ __forceinline__ bool mag_at_least_2m60(double x)
{
    const unsigned long long m = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    return m >= 0x3C30000000000000ull && m < 0x7ff0000000000000ull;
}

// True when hllc's outputs are certainly finite, from its inputs and its speeds: every side value
// finite and at most 2^60 in magnitude, and each divisor hllc forms -- S_L - S_P and S_R - S_P (the
// star ratios) and S_L - u_L, S_R - u_R (the star energies) -- at least 2^-60 in magnitude; its
// contact-speed divisor is clamped to at least 1e-20. Then |S_L|, |S_R| <= 2^61, |S_P| < 2^251, the
// ratios are below 2^122, the star energies below 2^563 and every flux component and u* below
// 2^750, far from overflow: no infinity, and so no NaN, can arise. False otherwise (the caller then
// forms the values).
__device__ __forceinline__ bool hllc_surely_finite(const Side<double> &L, const Side<double> &R, double SL, double SR,
                                                   double SP)
{
    bool ok = true;
    const double v[18] = {L.ar1, L.ar2, L.rho, L.un, L.ut, L.p, L.a, L.c, L.E,
                          R.ar1, R.ar2, R.rho, R.un, R.ut, R.p, R.a, R.c, R.E};
#pragma unroll
    for (int k = 0; k < 18; ++k) ok = ok && mag_at_most_2p60(v[k]);
    return ok && mag_at_least_2m60(SL - L.un) && mag_at_least_2m60(SR - R.un) && mag_at_least_2m60(SL - SP) &&
           mag_at_least_2m60(SR - SP);
}

template <int DIR, bool LAZY_E = false, typename T>
__device__ __forceinline__ void hllc(const Side<T> &L, const Side<T> &R, T f[6], T &ustar)
{
    constexpr int N = DIR == 0 ? 2 : 3;  // normal momentum component
    constexpr int Tc = DIR == 0 ? 3 : 2; // tangential momentum component
    T SL, SR, SP;
    hllc_speeds(L, R, SL, SR, SP);
    T ratioL, ratioR;
    sw_div2(SL - L.un, SL - SP, SR - R.un, SR - SP, ratioL, ratioR);
    T EL = L.E, ER = R.E;
    if constexpr (LAZY_E) {
        const bool left = fpos(SL) || (fle(SL, T(0)) && fpos(SP));
        const T rho = left ? L.rho : R.rho, un = left ? L.un : R.un, ut = left ? L.ut : R.ut;
        const T p = left ? L.p : R.p, gb = left ? L.gb : R.gb, pb = left ? L.pb : R.pb;
        EL = ER = gb * p + pb + T(0.5) * rho * (un * un + ut * ut);
    }

    // The flux of the region the contact and wave speeds put the face in (SC:594-662): left
    // supersonic (SL > 0), left star (SL <= 0 < SP), right star (SP <= 0 <= SR) or right supersonic
    // (the rest, NaN cases included) -- formed from the one side K it reads, selected bit for bit,
    // with the star correction S_K (U*_K - U_K) where the side is subsonic: the regions' expressions,
    // without evaluating the other side's.
    const bool b1 = fpos(SL);
    const bool b2 = !b1 && fle(SL, T(0)) && fpos(SP);
    const bool b3 = !b1 && !b2 && fle(SP, T(0)) && fle(T(0), SR);
    const bool left = b1 || b2, star = b2 || b3;
    const T ar1 = left ? L.ar1 : R.ar1, ar2 = left ? L.ar2 : R.ar2, rho = left ? L.rho : R.rho;
    const T un = left ? L.un : R.un, ut = left ? L.ut : R.ut, p = left ? L.p : R.p, a = left ? L.a : R.a;
    const T EK = left ? EL : ER;
    if (star) {
        const T S = left ? SL : SR, ratio = left ? ratioL : ratioR;
        const T E_star = EK + (SP - un) * (SP * rho + sw_div(p, S - un));
        f[0] = ar1 * un + S * (ar1 * ratio - ar1);
        f[1] = ar2 * un + S * (ar2 * ratio - ar2);
        f[N] = (rho * un * un + p) + S * (rho * SP * ratio - rho * un);
        f[Tc] = (rho * un * ut) + S * (rho * ut * ratio - rho * ut);
        f[4] = (EK + p) * un + S * (E_star * ratio - EK);
        f[5] = a * un + S * (a * ratio - a);
    } else {
        f[0] = ar1 * un;
        f[1] = ar2 * un;
        f[N] = rho * un * un + p;
        f[Tc] = rho * un * ut;
        f[4] = (EK + p) * un;
        f[5] = a * un;
    }
    T left_part = L.un + wmin(T(0), SL) * (ratioL - T(1));
    T right_part = R.un + wmax(T(0), SR) * (ratioR - T(1));
    T sp_sign = wsign(SP);
    ustar = sign_select(sp_sign, left_part, right_part);
}

// Blend of a high-order face value toward the first-order one, low + theta (high - low)
// (pp_blend_*_flux_kernel body, SC:1506-1512), with one deliberate difference in binary64: at
// theta = 1 with a finite low value it is the high value itself -- the blend's exact value, where
// the reference's low + (high - low) can round one unit away -- so a face the limiter leaves alone
// keeps its high-order flux and the in-place blend need not rewrite it. A non-finite low, high or theta
// takes the formula (NaN propagates as in the reference). Shared by the in-place limiter and the
// fused stage so both give the same bits. The tests are integer compares of the bit patterns.
__device__ __forceinline__ bool is_one(double t) { return __double_as_longlong(t) == 0x3ff0000000000000LL; }
__device__ __forceinline__ bool is_one(float t) { return __float_as_uint(t) == 0x3f800000u; }
__device__ __forceinline__ bool finite_bits(double x)
{
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) < 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool finite_bits(float x) { return (__float_as_uint(x) & 0x7fffffffu) < 0x7f800000u; }
__device__ __forceinline__ double face_blend(double low, double high, double theta)
{
    return is_one(theta) && finite_bits(low) ? high : __fma_rn(theta, high - low, low);
}
// Binary32 (the precision form's rebuilt blends): the reference's formula. The theta = 1 rule with
// the first-order finiteness bytes was measured slower there (triple point 2604 -> 2325
// Mcell-stage/s): the latency-bound rebuilt blends then wait on the byte before the first-order
// load, which costs more than the 4-byte loads it saves.
__device__ __forceinline__ float face_blend(float low, float high, float theta)
{
    return __fmaf_rn(theta, high - low, low);
}
// True when face_blend(low, high, theta) is `high` for every component of a face whose first-order
// values are all finite (`lofin`, the sweep's per-face byte): the binary64 blend at theta = 1 then
// needs no first-order value. Binary32 always blends.
__device__ __forceinline__ bool keeps_high(double theta, bool lofin) { return lofin && is_one(theta); }
__device__ __forceinline__ bool keeps_high(float, bool) { return false; }

// Flux difference terms with their rounding pinned (explicit fused multiply-add and products, which
// the compiler does not re-associate or contract): every kernel that forms a residual or a limiter
// state -- in-place or rebuilt blends, per-solve or batched -- rounds it the same way.
__device__ __forceinline__ double div_sum(double dfx, double idx, double dgy, double idy)
{
    return __fma_rn(dfx, idx, __dmul_rn(dgy, idy));  // dfx / dx + dgy / dy
}
__device__ __forceinline__ float div_sum(float dfx, float idx, float dgy, float idy)
{
    return __fmaf_rn(dfx, idx, __fmul_rn(dgy, idy));
}
__device__ __forceinline__ double src_term(double a, double d, double id)
{
    return __dmul_rn(__dmul_rn(a, d), id);  // a * d / dx
}
__device__ __forceinline__ float src_term(float a, float d, float id) { return __fmul_rn(__fmul_rn(a, d), id); }

}  // namespace wm
