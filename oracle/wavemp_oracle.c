/*
 * wavemp_oracle.c -- CPU restatement (FP64) of the reference's per-stage right-hand side.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle that the CUDA path is checked against and the
 * timed CPU baseline; the product never links, loads or calls it.
 *
 * It restates, function by function and in the same floating-point order of operations, the
 * Warp device functions and kernels of the reference scripts
 *   SC  = sainath_SC_it_works.py   (MUSCL + central-4 shear gated by a Ducros sensor, THINC)
 *   M10 = Sainath_M10.py           (THINC on the interface field always, staged Wong limiter on
 *                                   reconstructed states, pressure floor; no Ducros sensor)
 * and the unused MP5 / central-6 functions of both scripts, which the "mp5c6" reconstruction
 * calls where the shipped kernels call MUSCL / central-4.
 *
 * Build: -O2 -ffp-contract=off -fno-fast-math (no fused multiply-add, IEEE binary64 everywhere),
 * -fopenmp (loops over cells are independent; the only reduction is a min, so results do not
 * depend on the thread count). Under those flags the results are bit-identical to the golden
 * vectors that tests/golden/make_golden.py produces by running the reference's own kernel source.
 *
 * Array layout (as in the reference): every field is a (nx+2g) x (ny+2g) C-order float64 array,
 * x index i first, y index j contiguous; interior cells are i in [g, g+nx), j in [g, g+ny).
 * An x-face array entry fx[i, j] is the face between cells i and i+1; gy[i, j] the face between
 * j and j+1.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "wavemp_oracle.h"

/* Constants of SC:44-70 (identical in M10:42-67). */
#define WTINY 1.0e-20
#define WEPSM 1.0e-20
#define WMP5C 4.0
#define WB2 (4.0 / 3.0)
#define WKAP (1.0 / 3.0)
#define W1o60 (1.0 / 60.0)
#define WBETA_THINC 1.8
#define WYUXIN (0.9 * 0.35 * 1.0e-2 / (1.0 - 0.9 * 0.35))
#define WTHINC_THRESH 0.35
#define WPP_RHO 1.0e-10
#define WPP_ALPHA 1.0e-10
#define WPP_CTILDE 1.0e-8
#define WPP_HS_RHO 1.0e-11
#define WPP_HS_ALPHA 1.0e-11
#define WPP_HS_CTILDE 1.0e-9
#define WSIGMA_SMOOTH 0.01
#define PRIM_ALPHA_FLOOR 1.0e-8 /* cons_to_prim clamp, SC:852-853 */

typedef struct {
    double v0, v1, v2, v3, v4, v5;
} s6;

/* Warp builtins for float64: min/max as a<b?a:b / a>b?a:b, sign(x) = x<0 ? -1 : +1. */
static inline double wmin(double a, double b) { return a < b ? a : b; }
static inline double wmax(double a, double b) { return a > b ? a : b; }
static inline double wsign(double x) { return x < 0.0 ? -1.0 : 1.0; }

/* ---------------------------------------------------------------- EOS (SC:83-110) ---------- */
static inline void mix_gamma_pibig(const orc_params *P, double a1, double *gb, double *pb)
{
    double a2 = 1.0 - a1;
    *gb = a1 / (P->g1 - 1.0) + a2 / (P->g2 - 1.0);
    *pb = a1 * P->g1 * P->p1 / (P->g1 - 1.0) + a2 * P->g2 * P->p2 / (P->g2 - 1.0);
}

static inline void mix_gamma_pinf(const orc_params *P, double a1, double *g, double *pi)
{
    double gb, pb;
    mix_gamma_pibig(P, a1, &gb, &pb);
    *g = 1.0 / gb + 1.0;
    *pi = (*g - 1.0) * pb / *g;
}

static inline double sound_speed(const orc_params *P, double rho, double p, double a1)
{
    double g, pi;
    mix_gamma_pinf(P, a1, &g, &pi);
    double val = g * (p + pi) / rho;
    if (val < WTINY) val = WTINY;
    return sqrt(val);
}

static inline double prim_to_energy(const orc_params *P, double ar1, double ar2, double u,
                                    double v, double p, double a1)
{
    double rho = ar1 + ar2;
    double gb, pb;
    mix_gamma_pibig(P, a1, &gb, &pb);
    return gb * p + pb + 0.5 * rho * (u * u + v * v);
}

/* ------------------------------------------------- positivity helpers (SC:112-292) -------- */
static inline double clamp01_pp(double a1)
{
    double a = a1;
    if (isnan(a)) a = WPP_ALPHA;
    if (a < WPP_ALPHA) a = WPP_ALPHA;
    if (a > 1.0 - WPP_ALPHA) a = 1.0 - WPP_ALPHA;
    return a;
}

static inline double pp_theta_lower(double base, double high, double floor_)
{
    double theta = 1.0;
    if (isnan(base) || isnan(high)) {
        theta = 0.0;
    } else if (high < floor_) {
        double denom = base - high;
        if (denom > WTINY)
            theta = (base - floor_) / denom;
        else
            theta = 0.0;
    }
    if (theta < 0.0) theta = 0.0;
    if (theta > 1.0) theta = 1.0;
    return theta;
}

static inline s6 blend_s6(s6 base, s6 high, double theta)
{
    s6 s;
    s.v0 = base.v0 + theta * (high.v0 - base.v0);
    s.v1 = base.v1 + theta * (high.v1 - base.v1);
    s.v2 = base.v2 + theta * (high.v2 - base.v2);
    s.v3 = base.v3 + theta * (high.v3 - base.v3);
    s.v4 = base.v4 + theta * (high.v4 - base.v4);
    s.v5 = base.v5 + theta * (high.v5 - base.v5);
    return s;
}

static inline double rho_ctilde2_sc(const orc_params *P, s6 s)
{
    double g, pi;
    mix_gamma_pinf(P, clamp01_pp(s.v5), &g, &pi);
    return (s.v4 + pi) / (g - 1.0);
}

static inline s6 pp_floor_pressure_state(const orc_params *P, s6 s)
{
    double a1 = clamp01_pp(s.v5);
    double g, pi;
    mix_gamma_pinf(P, a1, &g, &pi);
    if (isnan(s.v4) || rho_ctilde2_sc(P, s) < WPP_CTILDE) s.v4 = WPP_CTILDE * (g - 1.0) - pi;
    s.v5 = a1;
    return s;
}

static inline s6 wong_stage_lower_s6(s6 base, s6 high, double base_val, double high_val,
                                     double floor_)
{
    double theta = 1.0;
    if (isnan(base_val) || isnan(high_val) || base_val < floor_) {
        theta = 0.0;
    } else if (high_val < floor_) {
        double denom = base_val - high_val;
        if (denom > WTINY)
            theta = (base_val - floor_) / denom;
        else
            theta = 0.0;
    }
    return blend_s6(base, high, theta);
}

/* SC:217-240 (called only by M10:1007-1008). */
static s6 pp_limit_reconstructed_state(const orc_params *P, s6 high, s6 base)
{
    s6 b = base;
    b.v5 = clamp01_pp(b.v5);
    if (b.v0 < WPP_RHO || isnan(b.v0)) b.v0 = WPP_RHO;
    if (b.v1 < WPP_RHO || isnan(b.v1)) b.v1 = WPP_RHO;

    s6 s = high;
    s = wong_stage_lower_s6(b, s, b.v0, s.v0, WPP_RHO);
    s = wong_stage_lower_s6(b, s, b.v1, s.v1, WPP_RHO);
    s = wong_stage_lower_s6(b, s, b.v5, s.v5, WPP_ALPHA);
    s = wong_stage_lower_s6(b, s, 1.0 - b.v5, 1.0 - s.v5, WPP_ALPHA);
    s = wong_stage_lower_s6(b, s, rho_ctilde2_sc(P, b), rho_ctilde2_sc(P, s), WPP_CTILDE);

    if (s.v0 < WPP_HS_RHO || s.v1 < WPP_HS_RHO || s.v5 < WPP_HS_ALPHA || s.v5 > 1.0 - WPP_HS_ALPHA)
        s = b;
    if (rho_ctilde2_sc(P, s) < WPP_HS_CTILDE || isnan(s.v4)) s = b;
    return s;
}

static inline double rho_ctilde2_cons(const orc_params *P, double m1, double m2, double mx,
                                      double my, double E, double a1_in)
{
    double a1 = clamp01_pp(a1_in);
    double mm1 = m1, mm2 = m2;
    if (mm1 < WPP_RHO || isnan(mm1)) mm1 = WPP_RHO;
    if (mm2 < WPP_RHO || isnan(mm2)) mm2 = WPP_RHO;
    double rho = mm1 + mm2;
    double uu = mx / rho;
    double vv = my / rho;
    double kin = 0.5 * rho * (uu * uu + vv * vv);
    double g, pi;
    mix_gamma_pinf(P, a1, &g, &pi);
    return E - kin - pi;
}

static inline double theta_cons_stage(const orc_params *P, const double l[6], const double h[6],
                                      int stage)
{
    double theta = 1.0;
    if (stage == 0) {
        theta = wmin(theta, pp_theta_lower(l[0], h[0], WPP_RHO));
        theta = wmin(theta, pp_theta_lower(l[1], h[1], WPP_RHO));
    } else if (stage == 1) {
        theta = wmin(theta, pp_theta_lower(l[5], h[5], WPP_ALPHA));
        theta = wmin(theta, pp_theta_lower(1.0 - l[5], 1.0 - h[5], WPP_ALPHA));
    } else {
        double lc = rho_ctilde2_cons(P, l[0], l[1], l[2], l[3], l[4], l[5]);
        double hc = rho_ctilde2_cons(P, h[0], h[1], h[2], h[3], h[4], h[5]);
        theta = pp_theta_lower(lc, hc, WPP_CTILDE);
    }
    if (theta < 0.0 || isnan(theta)) theta = 0.0;
    if (theta > 1.0) theta = 1.0;
    return theta;
}

/* ------------------------------------------------------------ limiters (SC:295-304) ------- */
static inline double mm2(double x, double y)
{
    return 0.5 * (wsign(x) + wsign(y)) * wmin(fabs(x), fabs(y));
}

static inline double mm4(double a, double b, double c, double d)
{
    double s = wsign(a) + wsign(b);
    return 0.125 * s * fabs((wsign(a) + wsign(c)) * (wsign(a) + wsign(d))) *
           wmin(wmin(fabs(a), fabs(b)), wmin(fabs(c), fabs(d)));
}

/* ------------------------------------------------------------ sensors (SC:308-325) -------- */
static inline double cell_entropy(const orc_params *P, double ar1, double ar2, double p, double a1)
{
    double rho = ar1 + ar2;
    if (rho < WTINY) rho = WTINY;
    double g, pi;
    mix_gamma_pinf(P, a1, &g, &pi);
    return p / pow(rho, g);
}

static inline double cator2_val(double em2, double em1, double e0, double ep1, double ep2)
{
    double aa = 0.25 * fabs(em2 - 4.0 * em1 + 3.0 * e0) + (13.0 / 12.0) * fabs(e0 - 2.0 * em1 + em2);
    double bb = 0.25 * fabs(3.0 * e0 - 4.0 * ep1 + ep2) + (13.0 / 12.0) * fabs(e0 - 2.0 * ep1 + ep2);
    return (2.0 * aa * bb + WYUXIN) / (aa * aa + bb * bb + WYUXIN);
}

/* ------------------------------------------------------ reconstructions (SC:327-446) ------- */
static inline double thinc_ul(double vm1, double v0, double v1)
{
    double result = v0;
    if ((v1 - v0) * (v0 - vm1) > 0.0) {
        double qa = 0.5 * (v1 + vm1);
        double qd = 0.5 * (v1 - vm1);
        double feng = (v0 - qa) / (qd);
        double T1 = tanh(WBETA_THINC * 0.5);
        double T2 = tanh(feng * WBETA_THINC * 0.5);
        result = qa + qd * (T1 + T2 / T1) / (1.0 + T2);
    }
    return result;
}

static inline double thinc_ur(double v0, double v1, double v2)
{
    double result = v1;
    if ((v2 - v1) * (v1 - v0) > 0.0) {
        double qa = 0.5 * (v2 + v0);
        double qd = 0.5 * (v2 - v0);
        double feng = (v1 - qa) / (qd);
        double T1 = tanh(WBETA_THINC * 0.5);
        double T2 = tanh(feng * WBETA_THINC * 0.5);
        result = qa - qd * (T1 - T2 / T1) / (1.0 - T2);
    }
    return result;
}

/* Suresh-Huynh MP5 as in SC:353-405; only the final (line 376 / 404) value is kept. */
static inline double mp5_ul(double vm2, double vm1, double v0, double vp1, double vp2)
{
    double VOR = W1o60 * (2.0 * vm2 - 13.0 * vm1 + 47.0 * v0 + 27.0 * vp1 - 3.0 * vp2);
    double VMP = v0 + mm2(vp1 - v0, WMP5C * (v0 - vm1));
    double result = VOR;
    if ((VOR - v0) * (VOR - VMP) >= WEPSM) {
        double DJM1 = vm2 - 2.0 * vm1 + v0;
        double DJ = vm1 - 2.0 * v0 + vp1;
        double DJP1 = v0 - 2.0 * vp1 + vp2;
        double DM4JPH = mm4(4.0 * DJ - DJP1, 4.0 * DJP1 - DJ, DJ, DJP1);
        double DM4JMH = mm4(4.0 * DJ - DJM1, 4.0 * DJM1 - DJ, DJ, DJM1);
        double VUL = v0 + WMP5C * (v0 - vm1);
        double VAV = 0.5 * (v0 + vp1);
        double VMD = VAV - 0.5 * DM4JPH;
        double VLC = v0 + 0.5 * (v0 - vm1) + WB2 * DM4JMH;
        double VMIN = wmax(wmin(wmin(v0, vp1), VMD), wmin(wmin(v0, VUL), VLC));
        double VMAX = wmin(wmax(wmax(v0, vp1), VMD), wmax(wmax(v0, VUL), VLC));
        result = VOR + mm2(VMIN - VOR, VMAX - VOR);
    }
    return result;
}

static inline double mp5_ur(double vm1, double v0, double vp1, double vp2, double vp3)
{
    double VOR = W1o60 * (-3.0 * vm1 + 27.0 * v0 + 47.0 * vp1 - 13.0 * vp2 + 2.0 * vp3);
    double VMP = vp1 + mm2(v0 - vp1, WMP5C * (vp1 - vp2));
    double result = VOR;
    if ((VOR - vp1) * (VOR - VMP) >= WEPSM) {
        double DJM1 = vm1 - 2.0 * v0 + vp1;
        double DJ = v0 - 2.0 * vp1 + vp2;
        double DJP1 = vp1 - 2.0 * vp2 + vp3;
        double DM4JPH = mm4(4.0 * DJ - DJP1, 4.0 * DJP1 - DJ, DJ, DJP1);
        double DM4JMH = mm4(4.0 * DJ - DJM1, 4.0 * DJM1 - DJ, DJ, DJM1);
        double VUL = vp1 + WMP5C * (vp1 - vp2);
        double VAV = 0.5 * (vp1 + v0);
        double VMD = VAV - 0.5 * DM4JMH;
        double VLC = vp1 + 0.5 * (vp1 - vp2) + WB2 * DM4JPH;
        double VMIN = wmax(wmin(wmin(vp1, v0), VMD), wmin(wmin(vp1, VUL), VLC));
        double VMAX = wmin(wmax(wmax(vp1, v0), VMD), wmax(wmax(vp1, VUL), VLC));
        result = VOR + mm2(VMIN - VOR, VMAX - VOR);
    }
    return result;
}

static inline double central6_avg(double vm2, double vm1, double v0, double vp1, double vp2,
                                  double vp3)
{
    double left = W1o60 * (2.0 * vm2 - 13.0 * vm1 + 47.0 * v0 + 27.0 * vp1 - 3.0 * vp2);
    double right = W1o60 * (-3.0 * vm1 + 27.0 * v0 + 47.0 * vp1 - 13.0 * vp2 + 2.0 * vp3);
    return 0.5 * (left + right);
}

static inline double central4(double wm1, double w0, double w1, double w2)
{
    /* SC:1076-1082 */
    return (-(1.0 / 12.0) * wm1 + (7.0 / 12.0) * w0 + (7.0 / 12.0) * w1 - (1.0 / 12.0) * w2);
}

static inline double muscl_char_ul(double vm1, double v0, double vp1, double vp2)
{
    (void)vp2;
    double dm = v0 - vm1;
    double d0 = vp1 - v0;
    return v0 + 0.25 * ((1.0 - WKAP) * mm2(dm, 2.0 * d0) + (1.0 + WKAP) * mm2(d0, 2.0 * dm));
}

static inline double muscl_char_ur(double vm1, double v0, double vp1, double vp2)
{
    (void)vm1;
    double dp = vp2 - vp1;
    double d0 = vp1 - v0;
    return vp1 - 0.25 * ((1.0 - WKAP) * mm2(dp, 2.0 * d0) + (1.0 + WKAP) * mm2(d0, 2.0 * dp));
}

/* ------------------------------------------------------ eigen-projections (SC:480-589) ----- */
static inline s6 to_char_x(s6 u, double c, double rho, double ar1, double ar2, double u_avg,
                           double v_avg)
{
    double inv2c = 0.5 / c;
    double inv2c2 = 0.5 / (c * c);
    double Y1 = ar1 / rho;
    double Y2 = ar2 / rho;
    double un = u_avg, ut = v_avg;
    s6 s;
    s.v0 = un * inv2c * u.v0 + un * inv2c * u.v1 - inv2c * u.v2 + inv2c2 * u.v4;
    s.v1 = u.v0 - Y1 / (c * c) * u.v4;
    s.v2 = u.v1 - Y2 / (c * c) * u.v4;
    s.v3 = -ut * u.v0 - ut * u.v1 + u.v3;
    s.v4 = u.v5;
    s.v5 = -un * inv2c * u.v0 - un * inv2c * u.v1 + inv2c * u.v2 + inv2c2 * u.v4;
    return s;
}

static inline s6 to_phys_x(s6 w, double c, double rho, double ar1, double ar2, double u_avg,
                           double v_avg)
{
    double c2 = c * c;
    double Y1 = ar1 / rho;
    double Y2 = ar2 / rho;
    s6 s;
    s.v0 = Y1 * (w.v0 + w.v5) + w.v1;
    s.v1 = Y2 * (w.v0 + w.v5) + w.v2;
    s.v2 = (u_avg - c) * w.v0 + u_avg * w.v1 + u_avg * w.v2 + (u_avg + c) * w.v5;
    s.v3 = v_avg * (w.v0 + w.v1 + w.v2 + w.v5) + w.v3;
    s.v4 = c2 * (w.v0 + w.v5);
    s.v5 = w.v4;
    return s;
}

static inline s6 to_char_y(s6 u, double c, double rho, double ar1, double ar2, double u_avg,
                           double v_avg)
{
    double inv2c = 0.5 / c;
    double inv2c2 = 0.5 / (c * c);
    double Y1 = ar1 / rho;
    double Y2 = ar2 / rho;
    double un = v_avg, ut_f = -u_avg;
    s6 s;
    s.v0 = un * inv2c * u.v0 + un * inv2c * u.v1 - inv2c * u.v3 + inv2c2 * u.v4;
    s.v1 = u.v0 - Y1 / (c * c) * u.v4;
    s.v2 = u.v1 - Y2 / (c * c) * u.v4;
    s.v3 = -ut_f * u.v0 - ut_f * u.v1 - u.v2;
    s.v4 = u.v5;
    s.v5 = -un * inv2c * u.v0 - un * inv2c * u.v1 + inv2c * u.v3 + inv2c2 * u.v4;
    return s;
}

static inline s6 to_phys_y(s6 w, double c, double rho, double ar1, double ar2, double u_avg,
                           double v_avg)
{
    double c2 = c * c;
    double Y1 = ar1 / rho;
    double Y2 = ar2 / rho;
    s6 s;
    s.v0 = Y1 * (w.v0 + w.v5) + w.v1;
    s.v1 = Y2 * (w.v0 + w.v5) + w.v2;
    s.v2 = u_avg * (w.v0 + w.v1 + w.v2 + w.v5) - w.v3;
    s.v3 = (v_avg - c) * w.v0 + v_avg * w.v1 + v_avg * w.v2 + (v_avg + c) * w.v5;
    s.v4 = c2 * (w.v0 + w.v5);
    s.v5 = w.v4;
    return s;
}

/* ------------------------------------------------------------- HLLC (SC:594-771) ----------- */
/* hllc_x and hllc_y differ only in which velocity is normal; `dir` selects the reference's
 * x (SC:594-662) or y (SC:690-752) formula, written out separately below where they differ. */
static s6 hllc(const orc_params *P, int dir, double ar1L, double ar2L, double uL, double vL,
               double pL, double a1L, double ar1R, double ar2R, double uR, double vR, double pR,
               double a1R)
{
    double rhoL = ar1L + ar2L;
    double rhoR = ar1R + ar2R;
    double cL = sound_speed(P, rhoL, pL, a1L);
    double cR = sound_speed(P, rhoR, pR, a1R);
    double EL = prim_to_energy(P, ar1L, ar2L, uL, vL, pL, a1L);
    double ER = prim_to_energy(P, ar1R, ar2R, uR, vR, pR, a1R);
    /* normal (n) and tangential (t) velocities */
    double nL = dir == 0 ? uL : vL, nR = dir == 0 ? uR : vR;

    double n_avg = 0.5 * (nL + nR);
    double c_avg = 0.5 * (cL + cR);
    double SL = wmin(nL - cL, n_avg - c_avg);
    double SR = wmax(nR + cR, n_avg + c_avg);

    double denom = rhoL * (SL - nL) - rhoR * (SR - nR);
    if (fabs(denom) < WTINY) denom = WTINY;
    double SP = (pR - pL + rhoL * nL * (SL - nL) - rhoR * nR * (SR - nR)) / denom;

    s6 f;
    if (SL > 0.0) {
        f.v0 = ar1L * nL;
        f.v1 = ar2L * nL;
        if (dir == 0) {
            f.v2 = rhoL * uL * uL + pL;
            f.v3 = rhoL * uL * vL;
        } else {
            f.v2 = rhoL * uL * vL;
            f.v3 = rhoL * vL * vL + pL;
        }
        f.v4 = (EL + pL) * nL;
        f.v5 = a1L * nL;
    } else if (SL <= 0.0 && 0.0 < SP) {
        double ratio = (SL - nL) / (SL - SP);
        double EL_star = EL + (SP - nL) * (SP * rhoL + pL / (SL - nL));
        double fL0 = ar1L * nL, fL1 = ar2L * nL;
        double fL2, fL3;
        if (dir == 0) {
            fL2 = rhoL * uL * uL + pL;
            fL3 = rhoL * uL * vL;
        } else {
            fL2 = rhoL * uL * vL;
            fL3 = rhoL * vL * vL + pL;
        }
        double fL4 = (EL + pL) * nL, fL5 = a1L * nL;
        f.v0 = fL0 + SL * (ar1L * ratio - ar1L);
        f.v1 = fL1 + SL * (ar2L * ratio - ar2L);
        if (dir == 0) {
            f.v2 = fL2 + SL * (rhoL * SP * ratio - rhoL * uL);
            f.v3 = fL3 + SL * (rhoL * vL * ratio - rhoL * vL);
        } else {
            f.v2 = fL2 + SL * (rhoL * uL * ratio - rhoL * uL);
            f.v3 = fL3 + SL * (rhoL * SP * ratio - rhoL * vL);
        }
        f.v4 = fL4 + SL * (EL_star * ratio - EL);
        f.v5 = fL5 + SL * (a1L * ratio - a1L);
    } else if (SP <= 0.0 && 0.0 <= SR) {
        double ratio = (SR - nR) / (SR - SP);
        double ER_star = ER + (SP - nR) * (SP * rhoR + pR / (SR - nR));
        double fR0 = ar1R * nR, fR1 = ar2R * nR;
        double fR2, fR3;
        if (dir == 0) {
            fR2 = rhoR * uR * uR + pR;
            fR3 = rhoR * uR * vR;
        } else {
            fR2 = rhoR * uR * vR;
            fR3 = rhoR * vR * vR + pR;
        }
        double fR4 = (ER + pR) * nR, fR5 = a1R * nR;
        f.v0 = fR0 + SR * (ar1R * ratio - ar1R);
        f.v1 = fR1 + SR * (ar2R * ratio - ar2R);
        if (dir == 0) {
            f.v2 = fR2 + SR * (rhoR * SP * ratio - rhoR * uR);
            f.v3 = fR3 + SR * (rhoR * vR * ratio - rhoR * vR);
        } else {
            f.v2 = fR2 + SR * (rhoR * uR * ratio - rhoR * uR);
            f.v3 = fR3 + SR * (rhoR * SP * ratio - rhoR * vR);
        }
        f.v4 = fR4 + SR * (ER_star * ratio - ER);
        f.v5 = fR5 + SR * (a1R * ratio - a1R);
    } else {
        f.v0 = ar1R * nR;
        f.v1 = ar2R * nR;
        if (dir == 0) {
            f.v2 = rhoR * uR * uR + pR;
            f.v3 = rhoR * uR * vR;
        } else {
            f.v2 = rhoR * uR * vR;
            f.v3 = rhoR * vR * vR + pR;
        }
        f.v4 = (ER + pR) * nR;
        f.v5 = a1R * nR;
    }
    return f;
}

/* Interface velocity u* for the non-conservative alpha source (SC:664-687 / 754-771).
 * nL, nR are the normal velocities. */
static double hllc_src(const orc_params *P, double ar1L, double ar2L, double nL, double pL,
                       double a1L, double ar1R, double ar2R, double nR, double pR, double a1R)
{
    double rhoL = ar1L + ar2L;
    double rhoR = ar1R + ar2R;
    double cL = sound_speed(P, rhoL, pL, a1L);
    double cR = sound_speed(P, rhoR, pR, a1R);
    double n_avg = 0.5 * (nL + nR);
    double c_avg = 0.5 * (cL + cR);
    double SL = wmin(nL - cL, n_avg - c_avg);
    double SR = wmax(nR + cR, n_avg + c_avg);
    double denom = rhoL * (SL - nL) - rhoR * (SR - nR);
    if (fabs(denom) < WTINY) denom = WTINY;
    double SP = (pR - pL + rhoL * nL * (SL - nL) - rhoR * nR * (SR - nR)) / denom;
    double left_part = nL + wmin(0.0, SL) * ((SL - nL) / (SL - SP) - 1.0);
    double right_part = nR + wmax(0.0, SR) * ((SR - nR) / (SR - SP) - 1.0);
    double sp_sign = wsign(SP);
    return 0.5 * (1.0 + sp_sign) * left_part + 0.5 * (1.0 - sp_sign) * right_part;
}

/* ================================================================ kernels ================= */
#define IDX(i, j) ((size_t)(i) * (size_t)nyg + (size_t)(j))

/* cons_to_prim_kernel, SC:840-864 (whole padded grid). */
void orc_cons_to_prim(const orc_params *P, int nxg, int nyg, double *ar1, double *ar2, double *ru,
                      double *rv, double *E, double *al, double *u_p, double *v_p, double *p_p)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nxg; ++i)
        for (int j = 0; j < nyg; ++j) {
            size_t k = IDX(i, j);
            double a1 = al[k];
            if (a1 < PRIM_ALPHA_FLOOR) a1 = PRIM_ALPHA_FLOOR;
            if (a1 > 1.0 - PRIM_ALPHA_FLOOR) a1 = 1.0 - PRIM_ALPHA_FLOOR;
            al[k] = a1;
            double rho = ar1[k] + ar2[k];
            double uu = ru[k] / rho;
            double vv = rv[k] / rho;
            double gb, pb;
            mix_gamma_pibig(P, a1, &gb, &pb);
            double pp = (E[k] - pb - 0.5 * rho * (uu * uu + vv * vv)) / gb;
            u_p[k] = uu;
            v_p[k] = vv;
            p_p[k] = pp;
        }
}

/* ducros_kernel, SC:875-916. */
void orc_ducros(int nxg, int nyg, const double *u_p, const double *v_p, const double *p_p,
                double *sigma_x, double *sigma_y)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nxg; ++i)
        for (int j = 0; j < nyg; ++j) {
            size_t k = IDX(i, j);
            if (i < 2 || i >= nxg - 2 || j < 2 || j >= nyg - 2) {
                sigma_x[k] = 1.0;
                sigma_y[k] = 1.0;
                continue;
            }
            double der_ux = 0.5 * (-u_p[IDX(i - 1, j)] + u_p[IDX(i + 1, j)]);
            double der_vx = 0.5 * (-v_p[IDX(i - 1, j)] + v_p[IDX(i + 1, j)]);
            double der_uy = 0.5 * (-u_p[IDX(i, j - 1)] + u_p[IDX(i, j + 1)]);
            double der_vy = 0.5 * (-v_p[IDX(i, j - 1)] + v_p[IDX(i, j + 1)]);
            double div_u = der_ux + der_vy;
            double curl_u = der_vx - der_uy;
            double ducros = div_u * div_u / (div_u * div_u + curl_u * curl_u + 1.0e-30);
            double pm2 = p_p[IDX(i - 2, j)], pm1 = p_p[IDX(i - 1, j)], p0 = p_p[k];
            double pp1 = p_p[IDX(i + 1, j)], pp2 = p_p[IDX(i + 2, j)];
            double aa = fabs(-pm2 + 16.0 * pm1 - 30.0 * p0 + 16.0 * pp1 - pp2);
            double bb = fabs(pm2 + 16.0 * pm1 + 30.0 * p0 + 16.0 * pp1 + pp2);
            sigma_x[k] = (aa / (bb + 1.0e-30)) * ducros;
            pm2 = p_p[IDX(i, j - 2)];
            pm1 = p_p[IDX(i, j - 1)];
            pp1 = p_p[IDX(i, j + 1)];
            pp2 = p_p[IDX(i, j + 2)];
            aa = fabs(-pm2 + 16.0 * pm1 - 30.0 * p0 + 16.0 * pp1 - pp2);
            bb = fabs(pm2 + 16.0 * pm1 + 30.0 * p0 + 16.0 * pp1 + pp2);
            sigma_y[k] = (aa / (bb + 1.0e-30)) * ducros;
        }
}

/* enforce_admissible_kernel, SC:918-958 (whole padded grid, in place). */
void orc_enforce_admissible(const orc_params *P, int nxg, int nyg, double *ar1, double *ar2,
                            double *ru, double *rv, double *E, double *al)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nxg; ++i)
        for (int j = 0; j < nyg; ++j) {
            size_t k = IDX(i, j);
            double a1 = clamp01_pp(al[k]);
            double m1 = ar1[k], m2 = ar2[k], mx = ru[k], my = rv[k];
            if (isnan(m1) || m1 < WPP_RHO) m1 = WPP_RHO;
            if (isnan(m2) || m2 < WPP_RHO) m2 = WPP_RHO;
            if (isnan(mx)) mx = 0.0;
            if (isnan(my)) my = 0.0;
            double rho = m1 + m2;
            double uu = mx / rho;
            double vv = my / rho;
            double kin = 0.5 * rho * (uu * uu + vv * vv);
            double gb, pb, g, pi;
            mix_gamma_pibig(P, a1, &gb, &pb);
            double p = (E[k] - pb - kin) / gb;
            mix_gamma_pinf(P, a1, &g, &pi);
            double p_min = WPP_CTILDE * (g - 1.0) - pi;
            if (isnan(E[k]) || isnan(p) || rho_ctilde2_cons(P, m1, m2, mx, my, E[k], a1) < WPP_CTILDE)
                E[k] = gb * p_min + pb + kin;
            ar1[k] = m1;
            ar2[k] = m2;
            ru[k] = mx;
            rv[k] = my;
            al[k] = a1;
        }
}

/* One face of fx_kernel / gy_kernel (SC:966-1301, M10:868-1222). `c(f, o)` reads field f of the
 * cell at offset o along the sweep (o = 0 is the left cell of the face). */
static void face_flux(const orc_params *P, int dir, const double *const cell[6],
                      const double *sigma, size_t k0, ptrdiff_t st, double out[7])
{
#define C(f, o) cell[f][(ptrdiff_t)k0 + (ptrdiff_t)(o) * st]
    s6 pm2 = {C(0, -2), C(1, -2), C(2, -2), C(3, -2), C(4, -2), C(5, -2)};
    s6 pm1 = {C(0, -1), C(1, -1), C(2, -1), C(3, -1), C(4, -1), C(5, -1)};
    s6 p0 = {C(0, 0), C(1, 0), C(2, 0), C(3, 0), C(4, 0), C(5, 0)};
    s6 pp1 = {C(0, 1), C(1, 1), C(2, 1), C(3, 1), C(4, 1), C(5, 1)};
    s6 pp2 = {C(0, 2), C(1, 2), C(2, 2), C(3, 2), C(4, 2), C(5, 2)};
    s6 pp3 = {C(0, 3), C(1, 3), C(2, 3), C(3, 3), C(4, 3), C(5, 3)};

    double e[8];
    for (int o = -3; o <= 4; ++o) e[o + 3] = cell_entropy(P, C(0, o), C(1, o), C(4, o), C(5, o));
    double c_m1 = cator2_val(e[0], e[1], e[2], e[3], e[4]);
    double c_0 = cator2_val(e[1], e[2], e[3], e[4], e[5]);
    double c_p1 = cator2_val(e[2], e[3], e[4], e[5], e[6]);
    double c_p2 = cator2_val(e[3], e[4], e[5], e[6], e[7]);
    int use_thinc = wmin(wmin(c_m1, c_0), wmin(c_p1, c_p2)) < WTHINC_THRESH;

    int use_smooth_shear = 0;
    if (P->variant == ORC_SC) {
        double smax = wmax(wmax(sigma[(ptrdiff_t)k0 - st], sigma[k0]),
                           wmax(sigma[(ptrdiff_t)k0 + st], sigma[(ptrdiff_t)k0 + 2 * st]));
        use_smooth_shear = smax < WSIGMA_SMOOTH;
    }
#undef C

    double ar1a = 0.5 * (p0.v0 + pp1.v0);
    double ar2a = 0.5 * (p0.v1 + pp1.v1);
    double a1a = 0.5 * (p0.v5 + pp1.v5);
    double pa = 0.5 * (p0.v4 + pp1.v4);
    double rhoa = ar1a + ar2a;
    double u_avg = 0.5 * (p0.v2 + pp1.v2) / rhoa;
    double v_avg = 0.5 * (p0.v3 + pp1.v3) / rhoa;
    double ca = sound_speed(P, rhoa, pa, a1a);

    s6 (*to_char)(s6, double, double, double, double, double, double) =
        dir == 0 ? to_char_x : to_char_y;
    s6 (*to_phys)(s6, double, double, double, double, double, double) =
        dir == 0 ? to_phys_x : to_phys_y;

    s6 wm2 = to_char(pm2, ca, rhoa, ar1a, ar2a, u_avg, v_avg);
    s6 wm1 = to_char(pm1, ca, rhoa, ar1a, ar2a, u_avg, v_avg);
    s6 w0 = to_char(p0, ca, rhoa, ar1a, ar2a, u_avg, v_avg);
    s6 w1 = to_char(pp1, ca, rhoa, ar1a, ar2a, u_avg, v_avg);
    s6 w2 = to_char(pp2, ca, rhoa, ar1a, ar2a, u_avg, v_avg);
    s6 w3 = to_char(pp3, ca, rhoa, ar1a, ar2a, u_avg, v_avg);

    double *wm2a = &wm2.v0, *wm1a = &wm1.v0, *w0a = &w0.v0, *w1a = &w1.v0, *w2a = &w2.v0,
           *w3a = &w3.v0;
    s6 wL, wR;
    double *wLa = &wL.v0, *wRa = &wR.v0;
    for (int f = 0; f < 6; ++f) {
        if (P->recon == ORC_MP5C6) {
            wLa[f] = mp5_ul(wm2a[f], wm1a[f], w0a[f], w1a[f], w2a[f]);
            wRa[f] = mp5_ur(wm1a[f], w0a[f], w1a[f], w2a[f], w3a[f]);
        } else {
            wLa[f] = muscl_char_ul(wm1a[f], w0a[f], w1a[f], w2a[f]);
            wRa[f] = muscl_char_ur(wm1a[f], w0a[f], w1a[f], w2a[f]);
        }
    }
    if (P->variant == ORC_SC) {
        if (use_smooth_shear) {
            double iph_v3 = P->recon == ORC_MP5C6
                                ? central6_avg(wm2.v3, wm1.v3, w0.v3, w1.v3, w2.v3, w3.v3)
                                : central4(wm1.v3, w0.v3, w1.v3, w2.v3);
            wL.v3 = iph_v3;
            wR.v3 = iph_v3;
        }
        if (use_thinc) {
            wL.v1 = thinc_ul(wm1.v1, w0.v1, w1.v1);
            wL.v2 = thinc_ul(wm1.v2, w0.v2, w1.v2);
            wL.v4 = thinc_ul(wm1.v4, w0.v4, w1.v4);
            wR.v1 = thinc_ur(w0.v1, w1.v1, w2.v1);
            wR.v2 = thinc_ur(w0.v2, w1.v2, w2.v2);
            wR.v4 = thinc_ur(w0.v4, w1.v4, w2.v4);
        }
    } else {
        if (use_thinc) {
            wL.v1 = thinc_ul(wm1.v1, w0.v1, w1.v1);
            wL.v2 = thinc_ul(wm1.v2, w0.v2, w1.v2);
        }
        wL.v4 = thinc_ul(wm1.v4, w0.v4, w1.v4);
        if (use_thinc) {
            wR.v1 = thinc_ur(w0.v1, w1.v1, w2.v1);
            wR.v2 = thinc_ur(w0.v2, w1.v2, w2.v2);
        }
        wR.v4 = thinc_ur(w0.v4, w1.v4, w2.v4);
    }

    s6 phL = to_phys(wL, ca, rhoa, ar1a, ar2a, u_avg, v_avg);
    s6 phR = to_phys(wR, ca, rhoa, ar1a, ar2a, u_avg, v_avg);
    s6 phfL = to_phys(w0, ca, rhoa, ar1a, ar2a, u_avg, v_avg);
    s6 phfR = to_phys(w1, ca, rhoa, ar1a, ar2a, u_avg, v_avg);

    if (P->variant == ORC_M10) {
        phL = pp_limit_reconstructed_state(P, phL, phfL);
        phR = pp_limit_reconstructed_state(P, phR, phfR);
    }
    if (phL.v0 < 0.0 || isnan(phL.v0)) phL.v0 = phfL.v0;
    if (phL.v1 < 0.0 || isnan(phL.v1)) phL.v1 = phfL.v1;
    if (phL.v5 < 0.0 || phL.v5 > 1.0) phL.v5 = phfL.v5;
    if (P->variant == ORC_M10) {
        if (rho_ctilde2_sc(P, phL) < WPP_CTILDE || isnan(phL.v4)) phL.v4 = phfL.v4;
        phL = pp_floor_pressure_state(P, phL);
    } else if (isnan(phL.v4)) {
        phL.v4 = phfL.v4;
    }
    if (phR.v0 < 0.0 || isnan(phR.v0)) phR.v0 = phfR.v0;
    if (phR.v1 < 0.0 || isnan(phR.v1)) phR.v1 = phfR.v1;
    if (phR.v5 < 0.0 || phR.v5 > 1.0) phR.v5 = phfR.v5;
    if (P->variant == ORC_M10) {
        if (rho_ctilde2_sc(P, phR) < WPP_CTILDE || isnan(phR.v4)) phR.v4 = phfR.v4;
        phR = pp_floor_pressure_state(P, phR);
    } else if (isnan(phR.v4)) {
        phR.v4 = phfR.v4;
    }
    if (ca < 0.0 || isnan(ca)) {
        phL = phfL;
        phR = phfR;
    }

    double rhoL = phL.v0 + phL.v1, rhoR = phR.v0 + phR.v1;
    double uL = phL.v2 / rhoL, vL = phL.v3 / rhoL;
    double uR = phR.v2 / rhoR, vR = phR.v3 / rhoR;
    s6 fl = hllc(P, dir, phL.v0, phL.v1, uL, vL, phL.v4, phL.v5, phR.v0, phR.v1, uR, vR, phR.v4,
                 phR.v5);
    double src = hllc_src(P, phL.v0, phL.v1, dir == 0 ? uL : vL, phL.v4, phL.v5, phR.v0, phR.v1,
                          dir == 0 ? uR : vR, phR.v4, phR.v5);
    out[0] = fl.v0;
    out[1] = fl.v1;
    out[2] = fl.v2;
    out[3] = fl.v3;
    out[4] = fl.v4;
    out[5] = fl.v5;
    out[6] = src;
}

/* fx_kernel (dir 0: faces i in [g-1, g+nx-1], rows j in [g, g+ny)) and gy_kernel (dir 1: columns
 * i in [g, g+nx), faces j in [g-1, g+ny-1]). cell = {ar1, ar2, ru, rv, p_p, al}. */
void orc_face_flux(const orc_params *P, int dir, int nx, int ny, int g, const double *const cell[6],
                   const double *sigma, double *const out[7])
{
    int nyg = ny + 2 * g;
    int i0 = dir == 0 ? g - 1 : g, i1 = dir == 0 ? g + nx : g + nx;
    int j0 = dir == 0 ? g : g - 1, j1 = dir == 0 ? g + ny : g + ny;
    ptrdiff_t st = dir == 0 ? (ptrdiff_t)nyg : 1;
#pragma omp parallel for schedule(static)
    for (int i = i0; i < i1; ++i)
        for (int j = j0; j < j1; ++j) {
            double f[7];
            size_t k = IDX(i, j);
            face_flux(P, dir, cell, sigma, k, st, f);
            for (int c = 0; c < 7; ++c) out[c][k] = f[c];
        }
}

/* fx_low_kernel / gy_low_kernel, SC:1303-1394. */
void orc_face_flux_low(const orc_params *P, int dir, int nx, int ny, int g,
                       const double *const cell[6], double *const out[7])
{
    int nyg = ny + 2 * g;
    int i0 = dir == 0 ? g - 1 : g, i1 = g + nx;
    int j0 = dir == 0 ? g : g - 1, j1 = g + ny;
    size_t st = dir == 0 ? (size_t)nyg : 1;
    const double *ar1 = cell[0], *ar2 = cell[1], *ru = cell[2], *rv = cell[3], *p_p = cell[4],
                 *al = cell[5];
#pragma omp parallel for schedule(static)
    for (int i = i0; i < i1; ++i)
        for (int j = j0; j < j1; ++j) {
            size_t kL = IDX(i, j), kR = kL + st;
            double rhoL = ar1[kL] + ar2[kL];
            double rhoR = ar1[kR] + ar2[kR];
            double uL = ru[kL] / rhoL, vL = rv[kL] / rhoL;
            double uR = ru[kR] / rhoR, vR = rv[kR] / rhoR;
            double aL = clamp01_pp(al[kL]), aR = clamp01_pp(al[kR]);
            double pL = p_p[kL], pR = p_p[kR];
            double gL, piL, gR, piR;
            mix_gamma_pinf(P, aL, &gL, &piL);
            mix_gamma_pinf(P, aR, &gR, &piR);
            if (isnan(pL) || (pL + piL) / (gL - 1.0) < WPP_CTILDE) pL = WPP_CTILDE * (gL - 1.0) - piL;
            if (isnan(pR) || (pR + piR) / (gR - 1.0) < WPP_CTILDE) pR = WPP_CTILDE * (gR - 1.0) - piR;
            s6 fl = hllc(P, dir, ar1[kL], ar2[kL], uL, vL, pL, aL, ar1[kR], ar2[kR], uR, vR, pR, aR);
            double src = hllc_src(P, ar1[kL], ar2[kL], dir == 0 ? uL : vL, pL, aL, ar1[kR],
                                  ar2[kR], dir == 0 ? uR : vR, pR, aR);
            out[0][kL] = fl.v0;
            out[1][kL] = fl.v1;
            out[2][kL] = fl.v2;
            out[3][kL] = fl.v3;
            out[4][kL] = fl.v4;
            out[5][kL] = fl.v5;
            out[6][kL] = src;
        }
}

/* pp_cell_theta_kernel, SC:1397-1476. q = {ar1, ar2, ru, rv, E, al}; fh/gh/fl/gl = 7 face
 * arrays each (6 fluxes + interface velocity). */
void orc_cell_theta(const orc_params *P, int nx, int ny, int g, const double *const q[6],
                    const double *al_prim, const double *const fh[7], const double *const gh[7],
                    const double *const fl[7], const double *const gl[7], double *theta_cell,
                    double dt, int stage)
{
    int nyg = ny + 2 * g;
    double inv_dx = 1.0 / P->dx, inv_dy = 1.0 / P->dy;
#pragma omp parallel for schedule(static)
    for (int i = g; i < g + nx; ++i)
        for (int j = g; j < g + ny; ++j) {
            size_t k = IDX(i, j), kx = IDX(i - 1, j), ky = IDX(i, j - 1);
            double a = al_prim[k];
            double rh[6], rl[6], l[6], h[6];
            for (int c = 0; c < 5; ++c) {
                rh[c] = (fh[c][k] - fh[c][kx]) * inv_dx + (gh[c][k] - gh[c][ky]) * inv_dy;
                rl[c] = (fl[c][k] - fl[c][kx]) * inv_dx + (gl[c][k] - gl[c][ky]) * inv_dy;
            }
            rh[5] = (fh[5][k] - fh[5][kx]) * inv_dx + (gh[5][k] - gh[5][ky]) * inv_dy -
                    a * (fh[6][k] - fh[6][kx]) * inv_dx - a * (gh[6][k] - gh[6][ky]) * inv_dy;
            rl[5] = (fl[5][k] - fl[5][kx]) * inv_dx + (gl[5][k] - gl[5][ky]) * inv_dy -
                    a * (fl[6][k] - fl[6][kx]) * inv_dx - a * (gl[6][k] - gl[6][ky]) * inv_dy;
            for (int c = 0; c < 6; ++c) {
                l[c] = q[c][k] - dt * rl[c];
                h[c] = q[c][k] - dt * rh[c];
            }
            theta_cell[k] = theta_cons_stage(P, l, h, stage);
        }
}

/* pp_blend_x_flux_kernel / pp_blend_y_flux_kernel, SC:1479-1548 (in place on fh). */
void orc_blend(int dir, int nx, int ny, int g, double *const fh[7], const double *const fl[7],
               const double *theta_cell)
{
    int nyg = ny + 2 * g;
    int i0 = dir == 0 ? g - 1 : g, i1 = g + nx;
    int j0 = dir == 0 ? g : g - 1, j1 = g + ny;
    size_t st = dir == 0 ? (size_t)nyg : 1;
#pragma omp parallel for schedule(static)
    for (int i = i0; i < i1; ++i)
        for (int j = j0; j < j1; ++j) {
            size_t k = IDX(i, j);
            int m = dir == 0 ? i : j, n = dir == 0 ? nx : ny;
            double theta = 1.0;
            if (m >= g && m < g + n) theta = wmin(theta, theta_cell[k]);
            if (m + 1 >= g && m + 1 < g + n) theta = wmin(theta, theta_cell[k + st]);
            for (int c = 0; c < 7; ++c) fh[c][k] = fl[c][k] + theta * (fh[c][k] - fl[c][k]);
        }
}

/* rk3_kernel, SC:1553-1611 (interior, in place on q). */
void orc_rk3(const orc_params *P, int nx, int ny, int g, const double *const q_old[6],
             double *const q[6], const double *al_prim, const double *const fx[7],
             const double *const gy[7], double dt, double alpha, double beta)
{
    int nyg = ny + 2 * g;
    double inv_dx = 1.0 / P->dx, inv_dy = 1.0 / P->dy;
#pragma omp parallel for schedule(static)
    for (int i = g; i < g + nx; ++i)
        for (int j = g; j < g + ny; ++j) {
            size_t k = IDX(i, j), kx = IDX(i - 1, j), ky = IDX(i, j - 1);
            double res[6];
            for (int c = 0; c < 5; ++c)
                res[c] = (fx[c][k] - fx[c][kx]) * inv_dx + (gy[c][k] - gy[c][ky]) * inv_dy;
            double src6x = al_prim[k] * (fx[6][k] - fx[6][kx]) * inv_dx;
            double src6y = al_prim[k] * (gy[6][k] - gy[6][ky]) * inv_dy;
            res[5] = (fx[5][k] - fx[5][kx]) * inv_dx + (gy[5][k] - gy[5][ky]) * inv_dy - src6x - src6y;
            for (int c = 0; c < 6; ++c) q[c][k] = alpha * q_old[c][k] + beta * (q[c][k] - dt * res[c]);
        }
}

/* Ghost fill. bc_x_kernel / bc_y_kernel, SC:1616-1682, generalised per side: kind 0 copies the
 * nearest interior cell (transmissive), kind 1 copies it and negates the wall-normal momentum and
 * velocity (the reference's slip wall). The x pass covers all rows, then the y pass all columns,
 * as in the reference. f9 = {ar1, ar2, ru, rv, E, al, u_p, v_p, p_p}. */
void orc_apply_bc(const int bc[4], int nx, int ny, int g, double *const f9[9])
{
    int nxg = nx + 2 * g, nyg = ny + 2 * g;
    for (int k = 0; k < g; ++k)
        for (int j = 0; j < nyg; ++j) {
            int li = g - 1 - k, ri = g + nx + k;
            for (int c = 0; c < 9; ++c) {
                double sl = f9[c][IDX(g, j)], sr = f9[c][IDX(g + nx - 1, j)];
                if (c == 2 || c == 6) {
                    if (bc[0] == 1) sl = -1.0 * sl;
                    if (bc[1] == 1) sr = -1.0 * sr;
                }
                f9[c][IDX(li, j)] = sl;
                f9[c][IDX(ri, j)] = sr;
            }
        }
    for (int i = 0; i < nxg; ++i)
        for (int k = 0; k < g; ++k) {
            int bj = g - 1 - k, tj = g + ny + k;
            for (int c = 0; c < 9; ++c) {
                double sb = f9[c][IDX(i, g)], st = f9[c][IDX(i, g + ny - 1)];
                if (c == 3 || c == 7) {
                    if (bc[2] == 1) sb = -1.0 * sb;
                    if (bc[3] == 1) st = -1.0 * st;
                }
                f9[c][IDX(i, bj)] = sb;
                f9[c][IDX(i, tj)] = st;
            }
        }
}

/* timestep_kernel + get_dt, SC:1686-1705, SC:1986-1995: CFL * min over interior cells. */
double orc_get_dt(const orc_params *P, int nx, int ny, int g, const double *ar1, const double *ar2,
                  const double *u_p, const double *v_p, const double *p_p, const double *al)
{
    int nyg = ny + 2 * g;
    double dtmin = 1.0e30;
#pragma omp parallel for schedule(static) reduction(min : dtmin)
    for (int i = g; i < g + nx; ++i)
        for (int j = g; j < g + ny; ++j) {
            size_t k = IDX(i, j);
            double rho = ar1[k] + ar2[k];
            double c = sound_speed(P, rho, p_p[k], al[k]);
            double sx = P->dx / (fabs(u_p[k]) + c);
            double sy = P->dy / (fabs(v_p[k]) + c);
            double dt_loc = sx * sy / (sx + sy);
            if (dt_loc < dtmin) dtmin = dt_loc;
        }
    return P->cfl * dtmin;
}

/* ============================================================ whole stage / step ========== */
/* ws holds 28 face arrays (fh 0..6, gh 0..6, fl 0..6, gl 0..6), theta, sigma_x, sigma_y and the
 * 6 old-state arrays, all of the padded grid size. */
size_t orc_workspace_doubles(int nx, int ny, int g)
{
    return (size_t)(28 + 3 + 6) * (size_t)(nx + 2 * g) * (size_t)(ny + 2 * g);
}

typedef struct {
    double *fh[7], *gh[7], *fl[7], *gl[7], *theta, *sx, *sy, *old[6];
} orc_ws;

static orc_ws split_ws(double *ws, int nx, int ny, int g)
{
    size_t n = (size_t)(nx + 2 * g) * (size_t)(ny + 2 * g);
    orc_ws w;
    for (int c = 0; c < 7; ++c) {
        w.fh[c] = ws + (size_t)c * n;
        w.gh[c] = ws + (size_t)(7 + c) * n;
        w.fl[c] = ws + (size_t)(14 + c) * n;
        w.gl[c] = ws + (size_t)(21 + c) * n;
    }
    w.theta = ws + 28 * n;
    w.sx = ws + 29 * n;
    w.sy = ws + 30 * n;
    for (int c = 0; c < 6; ++c) w.old[c] = ws + (size_t)(31 + c) * n;
    return w;
}

/* One SSP-RK3 stage in the reference's order (SC:2028-2055 body): apply_bc, compute_fluxes,
 * compute_low_fluxes, limit_fluxes, rk3_update, enforce_admissible, update_prims.
 * f10 = {ar1, ar2, ru, rv, E, al, u_p, v_p, p_p, al_prim}; q_old = 6 arrays. */
void orc_stage(const orc_params *P, int nx, int ny, int g, double *const f10[10],
               const double *const q_old[6], double *ws, double dt, double alpha, double beta)
{
    int nxg = nx + 2 * g, nyg = ny + 2 * g;
    orc_ws w = split_ws(ws, nx, ny, g);
    orc_apply_bc(P->bc, nx, ny, g, f10);
    const double *cell[6] = {f10[0], f10[1], f10[2], f10[3], f10[8], f10[5]};
    if (P->variant == ORC_SC) orc_ducros(nxg, nyg, f10[6], f10[7], f10[8], w.sx, w.sy);
    orc_face_flux(P, 0, nx, ny, g, cell, w.sx, w.fh);
    orc_face_flux(P, 1, nx, ny, g, cell, w.sy, w.gh);
    orc_face_flux_low(P, 0, nx, ny, g, cell, w.fl);
    orc_face_flux_low(P, 1, nx, ny, g, cell, w.gl);
    const double *q[6] = {f10[0], f10[1], f10[2], f10[3], f10[4], f10[5]};
    for (int s = 0; s < 3; ++s) {
        orc_cell_theta(P, nx, ny, g, q, f10[9], (const double *const *)w.fh,
                       (const double *const *)w.gh, (const double *const *)w.fl,
                       (const double *const *)w.gl, w.theta, dt, s);
        orc_blend(0, nx, ny, g, w.fh, (const double *const *)w.fl, w.theta);
        orc_blend(1, nx, ny, g, w.gh, (const double *const *)w.gl, w.theta);
    }
    orc_rk3(P, nx, ny, g, q_old, f10, f10[9], (const double *const *)w.fh,
            (const double *const *)w.gh, dt, alpha, beta);
    if (P->repair) orc_enforce_admissible(P, nxg, nyg, f10[0], f10[1], f10[2], f10[3], f10[4], f10[5]);
    orc_cons_to_prim(P, nxg, nyg, f10[0], f10[1], f10[2], f10[3], f10[4], f10[5], f10[6], f10[7],
                     f10[8]);
    memcpy(f10[9], f10[5], sizeof(double) * (size_t)nxg * (size_t)nyg);
}

/* `nsteps` SSP-RK3 steps (SC:2018-2059 minus save-time clamping and I/O): copy_old, three stages
 * with (alpha, beta) = (0, 1), (3/4, 1/4), (1/3, 2/3), then get_dt. *dt is the step's dt on entry
 * and the next dt on return. */
void orc_steps(const orc_params *P, int nx, int ny, int g, double *const f10[10], double *ws,
               int nsteps, double *dt)
{
    size_t n = (size_t)(nx + 2 * g) * (size_t)(ny + 2 * g);
    orc_ws w = split_ws(ws, nx, ny, g);
    for (int s = 0; s < nsteps; ++s) {
        for (int c = 0; c < 6; ++c) memcpy(w.old[c], f10[c], sizeof(double) * n);
        const double *old[6] = {w.old[0], w.old[1], w.old[2], w.old[3], w.old[4], w.old[5]};
        orc_stage(P, nx, ny, g, f10, old, ws, *dt, 0.0, 1.0);
        orc_stage(P, nx, ny, g, f10, old, ws, *dt, 0.75, 0.25);
        orc_stage(P, nx, ny, g, f10, old, ws, *dt, 1.0 / 3.0, 2.0 / 3.0);
        *dt = orc_get_dt(P, nx, ny, g, f10[0], f10[1], f10[6], f10[7], f10[8], f10[5]);
    }
}

/* Initialisation sequence of main(), SC:1998-2007 minus I/O. */
void orc_init_sequence(const orc_params *P, int nx, int ny, int g, double *const f10[10])
{
    int nxg = nx + 2 * g, nyg = ny + 2 * g;
    if (P->repair) orc_enforce_admissible(P, nxg, nyg, f10[0], f10[1], f10[2], f10[3], f10[4], f10[5]);
    orc_apply_bc(P->bc, nx, ny, g, f10);
    orc_cons_to_prim(P, nxg, nyg, f10[0], f10[1], f10[2], f10[3], f10[4], f10[5], f10[6], f10[7],
                     f10[8]);
    memcpy(f10[9], f10[5], sizeof(double) * (size_t)nxg * (size_t)nyg);
    orc_apply_bc(P->bc, nx, ny, g, f10);
}

/* ==================================================== single-function known-answer entry ==== */
/* Evaluates one device function on n packed input rows; used by the tests to pin the oracle
 * against vectors produced by the reference's own functions. Returns 0, or -1 for an unknown id. */
int orc_unit(const orc_params *P, int fn, long n, const double *in, int in_stride, double *out,
             int out_stride)
{
    for (long r = 0; r < n; ++r) {
        const double *a = in + r * in_stride;
        double *o = out + r * out_stride;
        switch (fn) {
        case ORC_FN_MP5_UL: o[0] = mp5_ul(a[0], a[1], a[2], a[3], a[4]); break;
        case ORC_FN_MP5_UR: o[0] = mp5_ur(a[0], a[1], a[2], a[3], a[4]); break;
        case ORC_FN_CENTRAL6: o[0] = central6_avg(a[0], a[1], a[2], a[3], a[4], a[5]); break;
        case ORC_FN_MUSCL_UL: o[0] = muscl_char_ul(a[0], a[1], a[2], a[3]); break;
        case ORC_FN_MUSCL_UR: o[0] = muscl_char_ur(a[0], a[1], a[2], a[3]); break;
        case ORC_FN_THINC_UL: o[0] = thinc_ul(a[0], a[1], a[2]); break;
        case ORC_FN_THINC_UR: o[0] = thinc_ur(a[0], a[1], a[2]); break;
        case ORC_FN_CATOR2: o[0] = cator2_val(a[0], a[1], a[2], a[3], a[4]); break;
        case ORC_FN_MM4: o[0] = mm4(a[0], a[1], a[2], a[3]); break;
        case ORC_FN_MM2: o[0] = mm2(a[0], a[1]); break;
        case ORC_FN_EOS: mix_gamma_pinf(P, a[0], &o[0], &o[1]); break;
        case ORC_FN_HLLC_X:
        case ORC_FN_HLLC_Y: {
            int dir = fn == ORC_FN_HLLC_Y;
            s6 f = hllc(P, dir, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10],
                        a[11]);
            o[0] = f.v0; o[1] = f.v1; o[2] = f.v2; o[3] = f.v3; o[4] = f.v4; o[5] = f.v5;
            o[6] = hllc_src(P, a[0], a[1], dir ? a[3] : a[2], a[4], a[5], a[6], a[7],
                            dir ? a[9] : a[8], a[10], a[11]);
            break;
        }
        case ORC_FN_EIGEN: {
            /* a = U[6], avg[6] (ar1, ar2, u, v, p, alpha); o = char_x, phys_x, char_y, phys_y */
            s6 U = {a[0], a[1], a[2], a[3], a[4], a[5]};
            double rho = a[6] + a[7];
            double c = sound_speed(P, rho, a[10], a[11]);
            s6 w = to_char_x(U, c, rho, a[6], a[7], a[8], a[9]);
            s6 b = to_phys_x(w, c, rho, a[6], a[7], a[8], a[9]);
            memcpy(o, &w, sizeof w);
            memcpy(o + 6, &b, sizeof b);
            w = to_char_y(U, c, rho, a[6], a[7], a[8], a[9]);
            b = to_phys_y(w, c, rho, a[6], a[7], a[8], a[9]);
            memcpy(o + 12, &w, sizeof w);
            memcpy(o + 18, &b, sizeof b);
            break;
        }
        case ORC_FN_PPLIM: {
            s6 h = {a[0], a[1], a[2], a[3], a[4], a[5]};
            s6 b = {a[6], a[7], a[8], a[9], a[10], a[11]};
            s6 s = pp_limit_reconstructed_state(P, h, b);
            memcpy(o, &s, sizeof s);
            break;
        }
        case ORC_FN_THETA: {
            for (int s = 0; s < 3; ++s) o[s] = theta_cons_stage(P, a, a + 6, s);
            break;
        }
        default: return -1;
        }
    }
    return 0;
}
