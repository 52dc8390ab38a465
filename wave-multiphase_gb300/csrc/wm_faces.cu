// wm_faces.cu -- face sweeps of the per-stage RHS: the high-order flux of fx_kernel / gy_kernel
// (SC:966-1301, M10:868-1222) and the first-order flux of fx_low_kernel / gy_low_kernel
// (SC:1303-1394) for one face per thread: binary64 in the plain form, binary32 in the precision
// form (which reads the binary32 cell copies and per-cell data of prep32_kernel).
//
// Per face: stencil load of six cells along the sweep, face-averaged eigenvectors, projection of
// the six cells to characteristic variables, MUSCL or MP5 / THINC / central reconstruction of the
// six fields, back-projection, positivity fallback (and for M10 the staged Wong limiter and the
// pressure floor), HLLC flux and interface velocity. The first-order flux reuses the per-cell
// state prepared by prep_kernel. Both results are written for the limiter.
#include "wm_kernels.cuh"

namespace wm {

namespace {

constexpr int FBX = 32, FBY = 4;

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

template <int DIR, int VAR, int REC, typename T, typename CS, typename FT>
__global__ void __launch_bounds__(FBX *FBY, 2)
face_kernel(Grid g, Eos e, CS cs, PrepT<T> p, Face<FT> hi, Face<FT> lo, int do_high, int do_low)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x + (DIR == 0 ? g.g : g.g - 1);
    const int i = blockIdx.y * blockDim.y + threadIdx.y + (DIR == 0 ? g.g - 1 : g.g);
    if (i >= g.g + g.nx || j >= g.g + g.ny) return;
    constexpr int N = DIR == 0 ? 2 : 3;   // normal momentum field
    constexpr int TG = DIR == 0 ? 3 : 2;  // tangential momentum field
    const long long sf = DIR == 0 ? cs.pitch() : 1;  // stride along the sweep, cell arrays
    const long long sw = DIR == 0 ? g.nyg : 1;       // stride along the sweep, workspace
    const long long kf = (long long)i * cs.pitch() + j;
    const long long kw = (long long)i * g.nyg + j;

    // Cells 0 and 1 of the face (i and i+1 along the sweep).
    T U0[6], U1[6];
    cs.load(kf, U0);
    cs.load(kf + sf, U1);

    if (do_low) {  // first-order HLLC of the two cell states (fx_low_kernel, SC:1303-1347)
        Side<T> L, R;
        const T *un = DIR == 0 ? p.lu : p.lv, *ut = DIR == 0 ? p.lv : p.lu;
        L.ar1 = U0[0]; L.ar2 = U0[1]; L.rho = U0[0] + U0[1];
        L.un = un[kw]; L.ut = ut[kw]; L.p = p.lp[kw]; L.a = p.la[kw]; L.c = p.lc[kw]; L.E = p.lE[kw];
        R.ar1 = U1[0]; R.ar2 = U1[1]; R.rho = U1[0] + U1[1];
        R.un = un[kw + sw]; R.ut = ut[kw + sw]; R.p = p.lp[kw + sw]; R.a = p.la[kw + sw];
        R.c = p.lc[kw + sw]; R.E = p.lE[kw + sw];
        T f[6], us;
        hllc<DIR>(L, R, f, us);
#pragma unroll
        for (int c = 0; c < 6; ++c) lo.f[c][kw] = FT(f[c]);
        lo.f[6][kw] = FT(us);
    }
    if (!do_high) return;

    // --- sensors (per-cell, computed by sensor_kernel) -------------------------------------------
    const T *ci = DIR == 0 ? p.cx : p.cy;
    const T c_m1 = ci[kw - sw], c_0 = ci[kw], c_p1 = ci[kw + sw], c_p2 = ci[kw + 2 * sw];
    const bool use_thinc = wmin(wmin(c_m1, c_0), wmin(c_p1, c_p2)) < T(kThincThresh);
    bool smooth = false;
    if (VAR == kSC) {
        const T *sg = DIR == 0 ? p.sx : p.sy;
        const T smax = wmax(wmax(sg[kw - sw], sg[kw]), wmax(sg[kw + sw], sg[kw + 2 * sw]));
        smooth = smax < T(kSigmaSmooth);
    }

    // --- face-averaged state and eigenvector basis (SC:1039-1048) ------------------------------
    const T ar1a = T(0.5) * (U0[0] + U1[0]);
    const T ar2a = T(0.5) * (U0[1] + U1[1]);
    const T a1a = T(0.5) * (U0[5] + U1[5]);
    const T pa = T(0.5) * (U0[4] + U1[4]);
    const T rhoa = ar1a + ar2a;
    const T irhoa = T(1) / rhoa;
    FaceBasis<T> b;
    b.u = T(0.5) * (U0[2] + U1[2]) * irhoa;
    b.v = T(0.5) * (U0[3] + U1[3]) * irhoa;
    const T ca = sound_speed_r(e, irhoa, pa, a1a);
    {
        const T ic = T(1) / ca;
        b.c = ca;
        b.c2 = ca * ca;
        b.inv2c = T(0.5) * ic;
        b.inv2c2 = T(0.5) * (ic * ic);
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
            cs.load(kf + (o - 2) * sf, u);
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
            wL[f] = mp5_ul(W[0][f], W[1][f], W[2][f], W[3][f], W[4][f]);
            wR[f] = mp5_ur(W[1][f], W[2][f], W[3][f], W[4][f], W[5][f]);
        } else {
            wL[f] = muscl_char_ul(W[1][f], W[2][f], W[3][f]);
            wR[f] = muscl_char_ur(W[2][f], W[3][f], W[4][f]);
        }
    }

    // --- back-projection and positivity fallback (SC:1095-1115; M10:1000-1025) ----------------
    S6<T> phL = to_phys<DIR>(b, wL), phR = to_phys<DIR>(b, wR);
    const S6<T> phfL = to_phys<DIR>(b, W[2]), phfR = to_phys<DIR>(b, W[3]);
    if (VAR == kM10) {
        phL = pp_limit_reconstructed_state(e, phL, phfL);
        phR = pp_limit_reconstructed_state(e, phR, phfR);
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        S6<T> &ph = s == 0 ? phL : phR;
        const S6<T> &pf = s == 0 ? phfL : phfR;
        if (ph.v[0] < T(0) || wisnan(ph.v[0])) ph.v[0] = pf.v[0];
        if (ph.v[1] < T(0) || wisnan(ph.v[1])) ph.v[1] = pf.v[1];
        if (ph.v[5] < T(0) || ph.v[5] > T(1)) ph.v[5] = pf.v[5];
        if (VAR == kM10) {
            if (rho_ctilde2_sc(e, ph) < T(kPpCtilde) || wisnan(ph.v[4])) ph.v[4] = pf.v[4];
            ph = pp_floor_pressure_state(e, ph);
        } else if (wisnan(ph.v[4])) {
            ph.v[4] = pf.v[4];
        }
    }
    if (ca < T(0) || wisnan(ca)) {
        phL = phfL;
        phR = phfR;
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
        const T ir = T(1) / d.rho;
        d.un = ph.v[N] * ir;
        d.ut = ph.v[TG] * ir;
        d.p = ph.v[4];
        d.a = ph.v[5];
        d.c = sound_speed_r(e, ir, d.p, d.a);
        d.E = prim_to_energy(e, d.rho, d.un, d.ut, d.p, d.a);
    }
    T f[6], us;
    hllc<DIR>(S[0], S[1], f, us);
#pragma unroll
    for (int c = 0; c < 6; ++c) hi.f[c][kw] = FT(f[c]);
    hi.f[6][kw] = FT(us);
}

template <int DIR, int VAR, int REC, typename T, typename CS, typename FT>
void launch_one(const Grid &g, const Eos &e, const CS &cs, const PrepT<T> &p, const Face<FT> &hi,
                const Face<FT> &lo, bool high, bool low, cudaStream_t s)
{
    const int nj = DIR == 0 ? g.ny : g.ny + 1, ni = DIR == 0 ? g.nx + 1 : g.nx;
    dim3 grid((nj + FBX - 1) / FBX, (ni + FBY - 1) / FBY);
    face_kernel<DIR, VAR, REC, T, CS, FT><<<grid, dim3(FBX, FBY), 0, s>>>(g, e, cs, p, hi, lo, high, low);
}

template <int VAR, int REC, typename T, typename CS, typename FT>
void launch_pair(const Grid &g, const Eos &e, const CS &cs, const PrepT<T> &p, const Face<FT> &fh,
                 const Face<FT> &gh, const Face<FT> &fl, const Face<FT> &gl, bool high, bool low,
                 cudaStream_t s)
{
    launch_one<0, VAR, REC, T>(g, e, cs, p, fh, fl, high, low, s);
    launch_one<1, VAR, REC, T>(g, e, cs, p, gh, gl, high, low, s);
}

template <typename T, typename CS, typename FT>
void dispatch(const Grid &g, const Eos &e, int variant, int recon, const CS &cs, const PrepT<T> &p,
              const Face<FT> &fh, const Face<FT> &gh, const Face<FT> &fl, const Face<FT> &gl,
              bool high, bool low, cudaStream_t s)
{
    if (variant == kSC && recon == kMuscl) launch_pair<kSC, kMuscl, T>(g, e, cs, p, fh, gh, fl, gl, high, low, s);
    if (variant == kSC && recon == kMp5) launch_pair<kSC, kMp5, T>(g, e, cs, p, fh, gh, fl, gl, high, low, s);
    if (variant == kM10 && recon == kMuscl) launch_pair<kM10, kMuscl, T>(g, e, cs, p, fh, gh, fl, gl, high, low, s);
    if (variant == kM10 && recon == kMp5) launch_pair<kM10, kMp5, T>(g, e, cs, p, fh, gh, fl, gl, high, low, s);
}

}  // namespace

void launch_faces(const Grid &g, const Eos &e, int variant, int recon, const Fields &q,
                  const Prep &p, const Face7 &fh, const Face7 &gh, const Face7 &fl, const Face7 &gl,
                  bool high, bool low, cudaStream_t s)
{
    dispatch<double>(g, e, variant, recon, Src64{q}, p, fh, gh, fl, gl, high, low, s);
}

void launch_faces32(const Grid &g, const Eos &e, int variant, int recon, const Cells32 &c,
                    const PrepT<float> &p, const Face<float> &fh, const Face<float> &gh,
                    const Face<float> &fl, const Face<float> &gl, bool high, bool low,
                    cudaStream_t s)
{
    dispatch<float>(g, e, variant, recon, Src32{c, g.nyg}, p, fh, gh, fl, gl, high, low, s);
}

}  // namespace wm
