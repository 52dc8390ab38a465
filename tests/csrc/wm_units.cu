// wm_units.cu -- test-only library: the binary64 face sweep's device functions (csrc/wm_device.cuh)
// applied row by row to the reference's known-answer vectors (tests/golden/units.npz), in the
// forms and with the argument order the sweep itself uses. Not part of libwavemp.so.
//
// wmt_unit(fn, n, in, in_stride, out, out_stride, eos[4], stream): rows of device doubles.
#include <cuda_runtime.h>

#include "wm_device.cuh"

using namespace wm;

enum {
    U_MP5_UL = 0, U_MP5_UR, U_CENTRAL6, U_MUSCL_UL, U_MUSCL_UR, U_THINC_UL, U_THINC_UR, U_CATOR2,
    U_MM4, U_MM2, U_EOS, U_HLLC_X, U_HLLC_Y, U_EIGEN, U_PPLIM, U_THETA, U_SIGN_SELECT, U_LOG1P_PC,
    U_EXPM1_PC, U_COUNT
};

// A side of the high-order Riemann problem, built as the sweep builds it from a back-projected
// state (ar1, ar2, normal / tangential velocity, p, alpha1).
__device__ Side<double> side_of(const Eos &e, double ar1, double ar2, double un, double ut, double p, double a)
{
    Side<double> d;
    d.ar1 = ar1;
    d.ar2 = ar2;
    d.rho = ar1 + ar2;
    const double ir = sw_rcp(d.rho);
    d.un = un;
    d.ut = ut;
    d.p = p;
    d.a = a;
    d.c = sound_speed_r<double, true>(e, ir, p, a);
    mix_gamma_pibig(e, a, d.gb, d.pb);
    d.E = 0.0;
    return d;
}

template <int DIR>
__device__ void hllc_row(const Eos &e, const double *a, double *o)
{
    // a = left (ar1, ar2, u, v, p, alpha1), right (the same)
    const double unL = DIR == 0 ? a[2] : a[3], utL = DIR == 0 ? a[3] : a[2];
    const double unR = DIR == 0 ? a[8] : a[9], utR = DIR == 0 ? a[9] : a[8];
    const Side<double> L = side_of(e, a[0], a[1], unL, utL, a[4], a[5]);
    const Side<double> R = side_of(e, a[6], a[7], unR, utR, a[10], a[11]);
    double f[6], us;
    hllc<DIR, true>(L, R, f, us);
    for (int c = 0; c < 6; ++c) o[c] = f[c];
    o[6] = us;
}

__global__ void unit_kernel(int fn, long long n, const double *in, int is, double *out, int os, Eos e)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const double *a = in + r * is;
    double *o = out + r * os;
    switch (fn) {
    case U_MP5_UL:  // mp5_ul(vm2, vm1, v0, vp1, vp2): the sweep's left value from cells -2..2
        o[0] = mp5_diff(a[2], a[3], a[1] - a[0], a[2] - a[1], a[3] - a[2], a[4] - a[3]);
        break;
    case U_MP5_UR:  // mp5_ur(vm1, v0, vp1, vp2, vp3): the right value, the mirrored stencil
        o[0] = mp5_diff(a[2], a[1], -(a[4] - a[3]), -(a[3] - a[2]), -(a[2] - a[1]), -(a[1] - a[0]));
        break;
    case U_CENTRAL6: o[0] = central6_avg<double>(a[0], a[1], a[2], a[3], a[4], a[5]); break;
    case U_MUSCL_UL: o[0] = muscl_char_ul<double>(a[0], a[1], a[2]); break;     // (vm1, v0, vp1, -)
    case U_MUSCL_UR: o[0] = muscl_char_ur<double>(a[1], a[2], a[3]); break;     // (-, v0, vp1, vp2)
    case U_THINC_UL: o[0] = thinc_ul<double>(e, a[0], a[1], a[2]); break;
    case U_THINC_UR: o[0] = thinc_ur<double>(e, a[0], a[1], a[2]); break;
    case U_CATOR2: o[0] = cator2_val<double>(a[0], a[1], a[2], a[3], a[4]); break;
    case U_MM4: o[0] = mm4<double>(a[0], a[1], a[2], a[3]); break;
    case U_MM2: o[0] = mm2<double>(a[0], a[1]); break;
    case U_EOS: mix_gamma_pinf<double, true>(e, a[0], o[0], o[1]); break;
    case U_HLLC_X: hllc_row<0>(e, a, o); break;
    case U_HLLC_Y: hllc_row<1>(e, a, o); break;
    case U_EIGEN: {
        // a = U (6 conserved-order values), the face average (ar1, ar2, u, v, p, alpha1), and the
        // reference's own characteristic values w_x (6), w_y (6) for the back-projections
        FaceBasis<double> b;
        const double rho = a[6] + a[7];
        const double ir = sw_rcp(rho);
        const double c = sound_speed_r<double, true>(e, ir, a[10], a[11]);
        const double ic = sw_rcp(c);
        b.c = c;
        b.c2 = c * c;
        b.inv2c = half_of(ic);
        b.inv2c2 = half_of(ic * ic);
        b.Y1 = a[6] * ir;
        b.Y2 = a[7] * ir;
        b.Y1c2 = b.Y1 * (ic * ic);
        b.Y2c2 = b.Y2 * (ic * ic);
        b.u = a[8];
        b.v = a[9];
        const S6<double> wx = to_char<0>(b, a), wy = to_char<1>(b, a);
        const S6<double> px = to_phys<0>(b, a + 12), py = to_phys<1>(b, a + 18);
        for (int k = 0; k < 6; ++k) {
            o[k] = wx.v[k];
            o[6 + k] = px.v[k];
            o[12 + k] = wy.v[k];
            o[18 + k] = py.v[k];
        }
        break;
    }
    case U_PPLIM: {
        S6<double> h, b;
        for (int k = 0; k < 6; ++k) {
            h.v[k] = a[k];
            b.v[k] = a[6 + k];
        }
        const S6<double> s = pp_limit_reconstructed_state(e, h, b);
        for (int k = 0; k < 6; ++k) o[k] = s.v[k];
        break;
    }
    case U_THETA:
        for (int s = 0; s < 3; ++s) o[s] = theta_cons_stage(e, a, a + 6, s);
        break;
    case U_LOG1P_PC: o[0] = (double)log1p_pc((float)a[0]); break;  // binary32 arguments, given exactly
    case U_EXPM1_PC: o[0] = (double)expm1_pc((float)a[0]); break;
    case U_SIGN_SELECT:  // the interface velocity's choice of side by wp.sign(SP) (SC:686, 770)
        o[0] = sign_select(wsign(a[0]), a[1], a[2]);
        break;
    default: break;
    }
}

// Values each function reads and writes per row (the strides must cover them).
static const int kIn[U_COUNT] = {5, 5, 6, 4, 4, 3, 3, 5, 4, 2, 1, 12, 12, 24, 12, 12, 3};
static const int kOut[U_COUNT] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 2, 7, 7, 24, 6, 3, 1};

extern "C" int wmt_unit(int fn, long long n, const double *in, int in_stride, double *out, int out_stride,
                        const double *eos4, void *stream)
{
    if (fn < 0 || fn >= U_COUNT || n < 0 || !in || !out || !eos4) return -1;
    if (in_stride < kIn[fn] || out_stride < kOut[fn]) return -1;
    if (n == 0) return 0;
    const Eos e = make_eos(eos4[0], eos4[1], eos4[2], eos4[3]);
    const int threads = 128;
    unit_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, (cudaStream_t)stream>>>(
        fn, n, in, in_stride, out, out_stride, e);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}
