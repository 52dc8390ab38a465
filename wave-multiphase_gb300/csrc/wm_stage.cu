// wm_stage.cu -- ghost fill, per-cell preparation, Wong limiter passes, RK3 combine with repair and
// primitive recovery, and the time-step reduction (sm_103a, binary64).
//
// Thread mapping: threadIdx.x runs along j (the contiguous axis of every array) so that each warp
// reads and writes 256-byte rows; blocks are 32 x 4 threads.
#include "wm_bodies.cuh"

namespace wm {

namespace {

constexpr int BX = 32, BY = 4;

// ------------------------------------------------------------------------------ ghost fill ----
// bc_x_kernel (SC:1616-1646) generalised per side; kind 1 negates the normal momentum and velocity.
__global__ void bc_x_kernel(Grid g, int bl, int br, Fields q, Fields old, int save)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int k = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= g.nyg || k >= g.g) return;
    int li = g.g - 1 - k, ri = g.g + g.nx + k;
    long long kl = kf_of(q, li, j), kr = kf_of(q, ri, j);
    long long sl = kf_of(q, g.g, j), sr = kf_of(q, g.g + g.nx - 1, j);
#pragma unroll
    for (int c = 0; c < 9; ++c) {
        double *a = q.f[c];
        if (save && c < 6) {  // copy_old of the ghost cells, before they are overwritten
            old.f[c][(long long)li * old.pitch + j] = a[kl];
            old.f[c][(long long)ri * old.pitch + j] = a[kr];
        }
        double vl = a[sl], vr = a[sr];
        if (c == F_RU || c == F_U) {
            if (bl == 1) vl = -1.0 * vl;
            if (br == 1) vr = -1.0 * vr;
        }
        a[kl] = vl;
        a[kr] = vr;
    }
}

// bc_y_kernel (SC:1650-1682); runs after the x pass, so corners take the y rule.
__global__ void bc_y_kernel(Grid g, int bb, int bt, Fields q, Fields old, int save)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (k >= g.g || i >= g.nxg) return;
    int bj = g.g - 1 - k, tj = g.g + g.ny + k;
    long long kb = kf_of(q, i, bj), kt = kf_of(q, i, tj);
    long long sb = kf_of(q, i, g.g), st = kf_of(q, i, g.g + g.ny - 1);
    bool save_here = save && i >= g.g && i < g.g + g.nx;  // corners were saved by the x pass
#pragma unroll
    for (int c = 0; c < 9; ++c) {
        double *a = q.f[c];
        if (save_here && c < 6) {
            old.f[c][(long long)i * old.pitch + bj] = a[kb];
            old.f[c][(long long)i * old.pitch + tj] = a[kt];
        }
        double vb = a[sb], vt = a[st];
        if (c == F_RV || c == F_V) {
            if (bb == 1) vb = -1.0 * vb;
            if (bt == 1) vt = -1.0 * vt;
        }
        a[kb] = vb;
        a[kt] = vt;
    }
}

// ------------------------------------------------------------------------- stage kernels ----
// Thin launch wrappers over the bodies of wm_bodies.cuh.
__global__ void __launch_bounds__(BX *BY) prep_kernel(Grid g, Eos e, Fields q, Prep p, int prechecks)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nxg || j >= g.nyg) return;
    prep_body(g, e, q, p, prechecks != 0, i, j);
}

__global__ void __launch_bounds__(BX *BY) sensor_kernel(Grid g, Eos e, Fields q, Prep p, int sc, int prechecks)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nxg || j >= g.nyg) return;
    sensor_body(g, e, q, p, sc, prechecks != 0, i, j);
}

// Pass STAGE of the limiter; NP = STAGE rebuilds the blends of the earlier passes in registers
// (fused stage), NP = 0 reads fh/gh as the in-place blend sweeps left them (closures).
// Resident blocks per SM the limiter passes are compiled for (128 threads a block): passes 0 and 1
// 16 (32 registers), pass 2 8 in binary64 with blends in place, where the rare cells that form the
// first-order values on demand spill rather than every cell losing warps (64 registers), 10 in
// binary32 (51), 6 for binary64 with deferred blends (85) -- the counts the passes had before.
template <int STAGE, typename FT, int NP>
constexpr int theta_min_blocks()
{
    return STAGE < 2 ? 16 : (sizeof(FT) == 4 ? 10 : (NP == 0 ? 8 : 6));
}

template <int STAGE, typename FT, int NP, int VERIFY = 0>
__global__ void __launch_bounds__(BX *BY, (theta_min_blocks<STAGE, FT, NP>()))
theta_kernel(Grid g, Eos e, Fields q, Cells32 c32, Face<FT> fh, Face<FT> gh, Face<FT> fl, Face<FT> gl,
             Theta3<FT> th3, double dt, const double *dt_dev, unsigned long long *limited,
             unsigned long long *verify, int prechecks)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x + g.g;
    int i = blockIdx.y * blockDim.y + threadIdx.y + g.g;
    if (i >= g.g + g.nx || j >= g.g + g.ny) return;
    if (dt_dev) dt = *dt_dev;
    double th = theta_body<STAGE, FT, NP, VERIFY, true>(g, e, q, c32, fh, gh, fl, gl, dt, th3.t, i, j,
                                                        verify, prechecks != 0);
    th3.t[STAGE][kw_of(g, i, j)] = store_as<FT>(th);
    if (limited) count_if(limited, flt(th, 1.0));
}

// Binary64: 16 resident blocks (32 registers). A face at theta = 1 reads its factor and byte only;
// the few at theta < 1 that form their first-order values on demand spill instead of every face
// losing warps.
template <typename FT>
__global__ void __launch_bounds__(BX *BY, (sizeof(FT) == 8 ? 16 : 1))
blend_kernel(Grid g, Face<FT> fh, Face<FT> gh, Face<FT> fl, Face<FT> gl, const FT *theta)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x + g.g - 1;
    int i = blockIdx.y * blockDim.y + threadIdx.y + g.g - 1;
    if (i >= g.g + g.nx || j >= g.g + g.ny) return;
    blend_body<FT, true>(g, fh, gh, fl, gl, theta, i, j);
}

template <typename FT, int NP>
__global__ void __launch_bounds__(BX *BY)
final_kernel(Grid g, Eos e, unsigned flags, Fields q, Fields old, Face<FT> fh, Face<FT> gh, Face<FT> fl,
             Face<FT> gl, Theta3<FT> th3, double dt, const double *dt_dev, double alpha, double beta, Counters cnt)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    unsigned long long dt_bits =
        final_body<FT, NP>(g, e, flags, q, old, fh, gh, fl, gl, th3.t, dt, dt_dev, alpha, beta, cnt, i, j);
    if (flags & FIN_DT) {
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long other = __shfl_down_sync(0xffffffffu, dt_bits, o);
            dt_bits = other < dt_bits ? other : dt_bits;
        }
        if ((threadIdx.x & 31) == 0 && dt_bits != ~0ull) atomicMin(cnt.dt_bits, dt_bits);
    }
}

// SW64: binary64 switches (a compile-time choice, so the binary32 sensor keeps its registers)
template <int SW64>
__global__ void __launch_bounds__(BX *BY) prep32_kernel(Grid g, Eos e, Fields q, PrepT<float> p, Cells32 c,
                                                        int prechecks)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nxg || j >= g.nyg) return;
    prep32_body(g, e, q, p, c, SW64 != 0, prechecks != 0, i, j);
}

template <int SW64>
__global__ void __launch_bounds__(BX *BY) sensor32_kernel(Grid g, Eos e, Fields q, PrepT<float> p, Cells32 c, int sc,
                                                          int prechecks)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nxg || j >= g.nyg) return;
    sensor32_body(g, e, q, p, c, sc, SW64 != 0, prechecks != 0, i, j);
}

// The THINC switch pre-check (thinc_side_pre on entropy32) and the binary64 decision (cator2_val of
// the binary64 entropies), both from the state, for the cell's x and y stencils.
__global__ void __launch_bounds__(BX *BY) switch_verify_kernel(Grid g, Eos e, Fields q, unsigned long long *verify)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nxg || j >= g.nyg) return;
    const long long kf = kf_of(q, i, j);
    for (int dir = 0; dir < 2; ++dir) {
        if (dir == 0 ? (i < 2 || i >= g.nxg - 2) : (j < 2 || j >= g.nyg - 2)) continue;
        const long long sq = dir == 0 ? q.pitch : 1;
        float s[5];
        double v[5];
        SwitchPairs w;  // the pairs prep stores, from the same binary64 values
        for (int k = 0; k < 5; ++k) {
            const long long c = kf + (k - 2) * sq;
            double gb, pb, ge, pie;
            mix_gamma_pibig(e, q.f[F_AL][c], gb, pb);
            entropy_gamma(gb, pb, ge, pie);
            double rho_e = q.f[F_AR1][c] + q.f[F_AR2][c];
            if (flt(rho_e, kTiny)) rho_e = kTiny;
            s[k] = entropy32(ge, rho_e, q.f[F_P][c]);
            v[k] = cell_entropy64(e, q, c);
            split32(q.f[F_P][c], w.v[PR_PH][k], w.v[PR_PL][k]);
            split32(rho_e, w.v[PR_RH][k], w.v[PR_RL][k]);
            split32(ge, w.v[PR_GH][k], w.v[PR_GL][k]);
        }
        // both pre-checks, in the sensor's order: binary32 entropies, then entropy ratios
        int d = thinc_side_pre(s[0], s[1], s[2], s[3], s[4]);
        if (d < 0) d = thinc_side_delta(w, s[2]);
        const float exact = side_of(cator2_val(v[0], v[1], v[2], v[3], v[4]), kThincThresh);
        count_if(&verify[0], true);
        count_if(&verify[1], d >= 0);
        count_if(&verify[2], d >= 0 && !(float(d) == exact));
    }
}

// The Ducros pre-check (ducros_pre on to_f32 of the state, the binary32 form's cell copies) and the
// binary64 decision (side_of of ducros_xy, the reference's sigma), for both directions of every cell
// with a full stencil.
__global__ void __launch_bounds__(BX *BY) ducros_verify_kernel(Grid g, Fields q, unsigned long long *verify)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < 2 || i >= g.nxg - 2 || j < 2 || j >= g.nyg - 2) return;
    const long long kf = kf_of(q, i, j);
    int dx, dy;
    ducros_pre(q.f[F_U], q.f[F_V], q.f[F_P], kf, q.pitch, 1, dx, dy);
    double sx, sy;
    ducros_xy(q, i, j, sx, sy);
    const float ex = side_of(sx, kSigmaSmooth), ey = side_of(sy, kSigmaSmooth);
    for (int dir = 0; dir < 2; ++dir) {
        const int d = dir == 0 ? dx : dy;
        const float exact = dir == 0 ? ex : ey;
        count_if(&verify[0], true);
        count_if(&verify[1], d >= 0);
        count_if(&verify[2], d >= 0 && !(float(d) == exact));
    }
}

__global__ void widen_kernel(const float *src, double *dst, long long n)
{
    long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k < n) dst[k] = double(src[k]);
}

__global__ void copy_old_kernel(Grid g, Fields q, Fields old)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nxg || j >= g.nyg) return;
    long long kf = kf_of(q, i, j), ko = (long long)i * old.pitch + j;
#pragma unroll
    for (int c = 0; c < 6; ++c) old.f[c][ko] = q.f[c][kf];
}

// timestep_kernel (SC:1686-1705) on the current primitives.
__global__ void dt_cell_kernel(Grid g, Eos e, Fields q, unsigned long long *dt_bits)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x + g.g;
    int i = blockIdx.y * blockDim.y + threadIdx.y + g.g;
    unsigned long long bits = ~0ull;
    if (i < g.g + g.nx && j < g.g + g.ny) {
        long long kf = kf_of(q, i, j);
        double rho = q.f[F_AR1][kf] + q.f[F_AR2][kf];
        // sx sy / (sx + sy) as one quotient, as the fused combine evaluates it (final_body)
        const double c = sound_speed_r<double, true>(e, rcp_nr(rho), q.f[F_P][kf], q.f[F_AL][kf]);
        const double d = div_nr(g.dx * g.dy, g.dy * (fabs(q.f[F_U][kf]) + c) + g.dx * (fabs(q.f[F_V][kf]) + c));
        bits = (unsigned long long)__double_as_longlong(d);
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long other = __shfl_down_sync(0xffffffffu, bits, o);
        bits = other < bits ? other : bits;
    }
    if ((threadIdx.x & 31) == 0 && bits != ~0ull) atomicMin(dt_bits, bits);
}

__global__ void dt_reset_kernel(unsigned long long *dt_bits)
{
    *dt_bits = (unsigned long long)__double_as_longlong(1.0e30);  // get_dt's initial value
}

__global__ void dt_finalize_kernel(const unsigned long long *dt_bits, double cfl, double *dt_out)
{
    *dt_out = cfl * __longlong_as_double((long long)*dt_bits);
}

__global__ void fp64_probe_kernel(double *out, int iters)
{
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
           x6 = x0 + 6, x7 = x0 + 7;
    const double a = 0.999999, b = 1e-7;
    for (int k = 0; k < iters; ++k) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

dim3 grid2(int nj, int ni) { return dim3((nj + BX - 1) / BX, (ni + BY - 1) / BY); }

}  // namespace

void launch_bc(const Grid &g, const int bc[4], const Fields &q, const Fields *save_old,
               cudaStream_t s)
{
    Fields old = save_old ? *save_old : q;
    int save = save_old != nullptr;
    bc_x_kernel<<<dim3((g.nyg + 63) / 64, g.g), dim3(64, 1), 0, s>>>(g, bc[0], bc[1], q, old, save);
    bc_y_kernel<<<dim3((g.g + 7) / 8, (g.nxg + 31) / 32), dim3(8, 32), 0, s>>>(g, bc[2], bc[3], q, old, save);
}

void launch_prep(const Grid &g, const Eos &e, const Fields &q, const Prep &p, int variant,
                 cudaStream_t s, bool prechecks)
{
    const int pc = prechecks ? 1 : 0;
    prep_kernel<<<grid2(g.nyg, g.nxg), dim3(BX, BY), 0, s>>>(g, e, q, p, pc);
    sensor_kernel<<<grid2(g.nyg, g.nxg), dim3(BX, BY), 0, s>>>(g, e, q, p, variant == kSC, pc);
}

template <typename FT>
void launch_limiter(const Grid &g, const Eos &e, const Fields &q, const Cells32 &c32, const Face<FT> &fh,
                    const Face<FT> &gh, const Face<FT> &fl, const Face<FT> &gl,
                    FT *const theta[3], double dt, const double *dt_dev, const Counters &cnt,
                    bool deferred, cudaStream_t s, unsigned long long *verify, bool prechecks)
{
    const dim3 gt = grid2(g.ny, g.nx), gb = grid2(g.ny + 1, g.nx + 1), bl(BX, BY);
    const Theta3<FT> t3{{theta[0], theta[1], theta[2]}};
    const int pc = prechecks ? 1 : 0;
    if (verify) {  // diagnostic: in-place blends, pre-check and binary64 solve both evaluated
        theta_kernel<0, FT, 0, 1><<<gt, bl, 0, s>>>(g, e, q, c32, fh, gh, fl, gl, t3, dt, dt_dev, nullptr, verify, pc);
        blend_kernel<FT><<<gb, bl, 0, s>>>(g, fh, gh, fl, gl, theta[0]);
        theta_kernel<1, FT, 0, 1><<<gt, bl, 0, s>>>(g, e, q, c32, fh, gh, fl, gl, t3, dt, dt_dev, nullptr, verify, pc);
        blend_kernel<FT><<<gb, bl, 0, s>>>(g, fh, gh, fl, gl, theta[1]);
        theta_kernel<2, FT, 0, 1><<<gt, bl, 0, s>>>(g, e, q, c32, fh, gh, fl, gl, t3, dt, dt_dev, nullptr, verify, pc);
        blend_kernel<FT><<<gb, bl, 0, s>>>(g, fh, gh, fl, gl, theta[2]);
        return;
    }
    if (deferred) {  // blends rebuilt by the next pass and by the combine
        theta_kernel<0, FT, 0><<<gt, bl, 0, s>>>(g, e, q, c32, fh, gh, fl, gl, t3, dt, dt_dev, cnt.limited, nullptr, pc);
        theta_kernel<1, FT, 1><<<gt, bl, 0, s>>>(g, e, q, c32, fh, gh, fl, gl, t3, dt, dt_dev, cnt.limited, nullptr, pc);
        theta_kernel<2, FT, 2><<<gt, bl, 0, s>>>(g, e, q, c32, fh, gh, fl, gl, t3, dt, dt_dev, cnt.limited, nullptr, pc);
        return;
    }
    theta_kernel<0, FT, 0><<<gt, bl, 0, s>>>(g, e, q, c32, fh, gh, fl, gl, t3, dt, dt_dev, cnt.limited, nullptr, pc);
    blend_kernel<FT><<<gb, bl, 0, s>>>(g, fh, gh, fl, gl, theta[0]);
    theta_kernel<1, FT, 0><<<gt, bl, 0, s>>>(g, e, q, c32, fh, gh, fl, gl, t3, dt, dt_dev, cnt.limited, nullptr, pc);
    blend_kernel<FT><<<gb, bl, 0, s>>>(g, fh, gh, fl, gl, theta[1]);
    theta_kernel<2, FT, 0><<<gt, bl, 0, s>>>(g, e, q, c32, fh, gh, fl, gl, t3, dt, dt_dev, cnt.limited, nullptr, pc);
    blend_kernel<FT><<<gb, bl, 0, s>>>(g, fh, gh, fl, gl, theta[2]);
}

template <typename FT>
void launch_final(const Grid &g, const Eos &e, unsigned flags, const Fields &q, const Fields &old,
                  const Face<FT> &fh, const Face<FT> &gh, const Face<FT> &fl, const Face<FT> &gl,
                  FT *const theta[3], bool deferred, double dt, const double *dt_dev,
                  double alpha, double beta, const Counters &cnt, cudaStream_t s)
{
    const Theta3<FT> t3{{theta[0], theta[1], theta[2]}};
    if (deferred && (flags & FIN_RK3))
        final_kernel<FT, 3><<<grid2(g.nyg, g.nxg), dim3(BX, BY), 0, s>>>(g, e, flags, q, old, fh, gh, fl, gl,
                                                                          t3, dt, dt_dev, alpha, beta, cnt);
    else
        final_kernel<FT, 0><<<grid2(g.nyg, g.nxg), dim3(BX, BY), 0, s>>>(g, e, flags, q, old, fh, gh, fl, gl,
                                                                          t3, dt, dt_dev, alpha, beta, cnt);
}

template void launch_limiter<double>(const Grid &, const Eos &, const Fields &, const Cells32 &,
                                     const Face<double> &, const Face<double> &, const Face<double> &,
                                     const Face<double> &, double *const[3], double, const double *,
                                     const Counters &, bool, cudaStream_t, unsigned long long *, bool);
template void launch_limiter<float>(const Grid &, const Eos &, const Fields &, const Cells32 &,
                                    const Face<float> &, const Face<float> &, const Face<float> &,
                                    const Face<float> &, float *const[3], double, const double *,
                                    const Counters &, bool, cudaStream_t, unsigned long long *, bool);
template void launch_final<double>(const Grid &, const Eos &, unsigned, const Fields &, const Fields &,
                                   const Face<double> &, const Face<double> &, const Face<double> &,
                                   const Face<double> &, double *const[3], bool, double, const double *,
                                   double, double, const Counters &, cudaStream_t);
template void launch_final<float>(const Grid &, const Eos &, unsigned, const Fields &, const Fields &,
                                  const Face<float> &, const Face<float> &, const Face<float> &,
                                  const Face<float> &, float *const[3], bool, double, const double *,
                                  double, double, const Counters &, cudaStream_t);

void launch_prep32(const Grid &g, const Eos &e, const Fields &q, const PrepT<float> &p,
                   const Cells32 &c, int variant, bool sw64, cudaStream_t s, bool prechecks)
{
    const int pc = prechecks ? 1 : 0;
    const dim3 grid = grid2(g.nyg, g.nxg), block(BX, BY);
    if (sw64) {
        prep32_kernel<1><<<grid, block, 0, s>>>(g, e, q, p, c, pc);
        sensor32_kernel<1><<<grid, block, 0, s>>>(g, e, q, p, c, variant == kSC, pc);
    } else {
        prep32_kernel<0><<<grid, block, 0, s>>>(g, e, q, p, c, pc);
        sensor32_kernel<0><<<grid, block, 0, s>>>(g, e, q, p, c, variant == kSC, pc);
    }
}

void launch_verify_switch(const Grid &g, const Eos &e, const Fields &q, unsigned long long *verify,
                          cudaStream_t s)
{
    switch_verify_kernel<<<grid2(g.nyg, g.nxg), dim3(BX, BY), 0, s>>>(g, e, q, verify);
}

void launch_verify_ducros(const Grid &g, const Fields &q, unsigned long long *verify, cudaStream_t s)
{
    ducros_verify_kernel<<<grid2(g.nyg, g.nxg), dim3(BX, BY), 0, s>>>(g, q, verify);
}

void launch_widen(const float *src, double *dst, long long n, cudaStream_t s)
{
    widen_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, n);
}

void launch_copy_old(const Grid &g, const Fields &q, const Fields &old, cudaStream_t s)
{
    copy_old_kernel<<<grid2(g.nyg, g.nxg), dim3(BX, BY), 0, s>>>(g, q, old);
}

void launch_dt_reset(const Counters &cnt, cudaStream_t s) { dt_reset_kernel<<<1, 1, 0, s>>>(cnt.dt_bits); }

void launch_dt_cell(const Grid &g, const Eos &e, const Fields &q, const Counters &cnt, cudaStream_t s)
{
    dt_cell_kernel<<<grid2(g.ny, g.nx), dim3(BX, BY), 0, s>>>(g, e, q, cnt.dt_bits);
}

void launch_dt_finalize(const Grid &g, const Counters &cnt, double *dt_out, cudaStream_t s)
{
    dt_finalize_kernel<<<1, 1, 0, s>>>(cnt.dt_bits, g.cfl, dt_out);
}

void launch_fp64_probe(double *out, int iters, cudaStream_t s, int blocks, int threads)
{
    fp64_probe_kernel<<<blocks, threads, 0, s>>>(out, iters);
}

}  // namespace wm
