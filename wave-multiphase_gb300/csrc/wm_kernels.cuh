// wm_kernels.cuh -- kernels of the per-stage RHS and their launch-argument blocks.
#pragma once
#include "wm_device.cuh"

namespace wm {

enum { kSC = 0, kM10 = 1 };
enum { kMuscl = 0, kMp5 = 1 };

// The ten per-cell arrays of the reference (ar1, ar2, ru, rv, E, al, u_p, v_p, p_p, al_prim).
struct Fields {
    double *f[10];
    long long pitch;
};
enum { F_AR1 = 0, F_AR2, F_RU, F_RV, F_E, F_AL, F_U, F_V, F_P, F_ALP };

// The inputs of the first-order flux of a face, for forming it on demand (the plain form's fused
// stage: the sweep writes only the finiteness bytes, and the limiter's bound solve and blends form
// the first-order values where they need them): the cells' partial densities (stage state, row
// pitch `pitch`) and the preparation pass's first-order cell states (padded-grid rows of nyg).
struct LowSrc {
    const double *ar1 = nullptr, *ar2 = nullptr;
    long long pitch = 0;
    const double *lu = nullptr, *lv = nullptr, *lp = nullptr, *la = nullptr, *lc = nullptr, *lE = nullptr;
    int nyg = 0;
    int on = 0;  // 1: the f arrays are not written; form the values from these inputs
};

// Six flux components and the interface velocity of one sweep direction; FT is the storage type
// (double in the plain form, float in the precision form). The first-order arrays also carry one
// byte per face, written by the sweep that writes them: 1 when all seven first-order values of the
// face are finite, else 0 -- what the limiter needs of a face it leaves unlimited (theta = 1), so
// that it need not read the seven values there.
template <typename FT> struct Face {
    FT *f[7];
    unsigned char *fin = nullptr;
};
template <> struct Face<double> {
    double *f[7];
    unsigned char *fin = nullptr;
    LowSrc src;  // first-order faces only: on-demand inputs (src.on = 1) instead of f
};
using Face7 = Face<double>;

// Per-cell data computed once per stage and shared by the faces that use it.
template <typename PT> struct PrepT {
    PT *ent;                          // cell entropy p / rho^gamma
    double *ent64;                    // the entropy in binary64 (plain form; precision form with
                                      // binary64 switches), every cell, when the pre-checks are off
    float *pair[6];                   // with the pre-checks: each cell's pressure, clamped density
                                      // and binary64 mixture gamma as binary32 pairs hi + lo
                                      // (PR_* order; the density pair overlays ent64)
    float *ent32;                     // the binary32 entropy of that pre-check (the precision
                                      // form's ent array, which its binary64 switches leave free)
    PT *cx, *cy;                      // smoothness indicator along x and y
    PT *sx, *sy;                      // Ducros x pressure sensor (SC only)
    PT *lu, *lv, *lp, *la, *lc, *lE;  // first-order HLLC cell state: velocity, floored
                                      // pressure, clamped alpha, sound speed, energy
};
using Prep = PrepT<double>;
// PrepT::pair: x = hi + lo with hi = x rounded to binary32, lo = the rest rounded (split32)
enum { PR_PH = 0, PR_PL, PR_RH, PR_RL, PR_GH, PR_GL };

// Places PrepT::pair in a workspace: the density pair in the binary64 entropy's slot (two binary32
// arrays of `cells` each, which the slot holds), the pressure and gamma pairs in consecutive
// binary32 arrays `stride` bytes apart from `next` -- the pressure hi first, unless `p_hi` (the
// precision form's binary32 pressure copy, the same values) is given: 4 arrays, or 3.
inline void set_pairs(float *pair[6], float *ent64_slot, size_t cells, char *next, size_t stride, float *p_hi)
{
    pair[PR_RH] = ent64_slot;
    pair[PR_RL] = ent64_slot + cells;
    int k = 0;
    auto take = [&]() { return reinterpret_cast<float *>(next + (size_t)(k++) * stride); };
    pair[PR_PH] = p_hi ? p_hi : take();
    pair[PR_PL] = take();
    pair[PR_GH] = take();
    pair[PR_GL] = take();
}

// Binary32 copies of the cell state read by the precision form's face sweep (workspace pitch).
struct Cells32 {
    float *ar1, *ar2, *ru, *rv, *p, *al, *u, *v;
    float *E;  // read by the limiter's binary32 pre-checks only
};

struct Counters {
    unsigned long long *repaired, *nonfinite, *limited;
    unsigned long long *dt_bits;  // atomic min of the positive dt candidates (bit pattern)
};

template <typename FT> struct Theta3 {
    FT *t[3];  // cell limiter factors of the three passes, in the flux type
};

// Flags of final_kernel.
enum : unsigned {
    FIN_RK3 = 1u,         // rk3_update on interior cells
    FIN_ADMISSIBLE = 2u,  // enforce_admissible on every cell
    FIN_PRIM = 4u,        // cons_to_prim + al_prim copy on every cell
    FIN_SAVE_OLD = 8u,    // copy the pre-update interior state to q_old (copy_old fused)
    FIN_DT = 16u,         // accumulate the time-step candidate of interior cells
    FIN_OLD_READ = 32u,   // rk3 reads q_old (alpha != 0)
    FIN_EXACT_CHECKS = 64u,  // precision form: no binary32 pre-check of the admissibility tests
};

void launch_bc(const Grid &g, const int bc[4], const Fields &q, const Fields *save_old,
               cudaStream_t s);
void launch_prep(const Grid &g, const Eos &e, const Fields &q, const Prep &p, int variant,
                 cudaStream_t s, bool prechecks = true);
void launch_faces(const Grid &g, const Eos &e, int variant, int recon, const Fields &q,
                  const Prep &p, const Face7 &fh, const Face7 &gh, const Face7 &fl, const Face7 &gl,
                  bool high, bool low, cudaStream_t s);
// The three limiter passes. deferred: no in-place blend sweeps -- each pass and the combine rebuild
// the blended fluxes in registers (bit-identical); fh/gh keep the unlimited high-order fluxes.
// c32: the binary32 cell copies of the precision form (its limiter pre-checks read them; unused
// for FT = double). verify: the pre-check diagnostic's two counters, or null.
template <typename FT>
void launch_limiter(const Grid &g, const Eos &e, const Fields &q, const Cells32 &c32, const Face<FT> &fh,
                    const Face<FT> &gh, const Face<FT> &fl, const Face<FT> &gl,
                    FT *const theta[3], double dt, const double *dt_dev, const Counters &cnt,
                    bool deferred, cudaStream_t s, unsigned long long *verify = nullptr,
                    bool prechecks = true);
template <typename FT>
void launch_final(const Grid &g, const Eos &e, unsigned flags, const Fields &q, const Fields &old,
                  const Face<FT> &fh, const Face<FT> &gh, const Face<FT> &fl, const Face<FT> &gl,
                  FT *const theta[3], bool deferred, double dt, const double *dt_dev,
                  double alpha, double beta, const Counters &cnt, cudaStream_t s);
void launch_copy_old(const Grid &g, const Fields &q, const Fields &old, cudaStream_t s);
void launch_dt_reset(const Counters &cnt, cudaStream_t s);
void launch_dt_cell(const Grid &g, const Eos &e, const Fields &q, const Counters &cnt,
                    cudaStream_t s);
void launch_dt_finalize(const Grid &g, const Counters &cnt, double *dt_out, cudaStream_t s);
void launch_fp64_probe(double *out, int iters, cudaStream_t s, int blocks, int threads);
// The THINC switch pre-check against the binary64 decision on every full stencil of q;
// verify[0..2]: stencils, decided by the pre-check, decided differently.
void launch_verify_switch(const Grid &g, const Eos &e, const Fields &q, unsigned long long *verify,
                          cudaStream_t s);
// The Ducros pre-check against the binary64 decision, both directions of every cell with a full
// stencil; verify[0..2] as launch_verify_switch.
void launch_verify_ducros(const Grid &g, const Fields &q, unsigned long long *verify, cudaStream_t s);

// Precision form (binary32 face sweep).
void launch_prep32(const Grid &g, const Eos &e, const Fields &q, const PrepT<float> &p,
                   const Cells32 &c, int variant, bool sw64, cudaStream_t s, bool prechecks = true);
void launch_faces32(const Grid &g, const Eos &e, int variant, int recon, const Cells32 &c,
                    const PrepT<float> &p, const Face<float> &fh, const Face<float> &gh,
                    const Face<float> &fl, const Face<float> &gl, bool high, bool low,
                    cudaStream_t s);
void launch_widen(const float *src, double *dst, long long n, cudaStream_t s);

}  // namespace wm
