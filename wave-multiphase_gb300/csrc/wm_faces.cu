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
#include "wm_bodies.cuh"

namespace wm {

namespace {

constexpr int FBX = 32, FBY = 4;

// Binary32 sweeps: registers capped for 8 resident blocks per SM (no spills; 64 registers instead
// of 89 lift the warp occupancy from 31 % to 50 % of the latency-bound kernel); binary64: 2.
template <int DIR, int VAR, int REC, typename T, typename CS, typename FT>
__global__ void __launch_bounds__(FBX *FBY, sizeof(T) == 4 ? 8 : 2)
face_kernel(Grid g, Eos e, CS cs, PrepT<T> p, Face<FT> hi, Face<FT> lo, int do_high, int do_low)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x + (DIR == 0 ? g.g : g.g - 1);
    const int i = blockIdx.y * blockDim.y + threadIdx.y + (DIR == 0 ? g.g - 1 : g.g);
    if (i >= g.g + g.nx || j >= g.g + g.ny) return;
    face_body<DIR, VAR, REC, T>(g, e, cs, p, hi, lo, do_high != 0, do_low != 0, i, j);
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
