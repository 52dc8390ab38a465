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

constexpr int FBX = 32, FBY = 4;  // faces of a block: FBY rows (x) by FBX columns (y, contiguous)
// Resident blocks per SM the binary64 sweep is compiled for: 4 fit its registers (128) without spills.
constexpr int kFace64Blocks = 4;

// A block's tile, staged in shared memory: the six cell fields over the block's faces and the
// stencil halo along the sweep (cells -2..3 of every face), the six first-order fields (cells 0, 1)
// and the two sensors (cells -1..2). Planes are (rows x columns) row-major; along x the tile has
// the block's FBX columns and FBY + 5 / + 1 / + 3 rows, along y FBY rows and FBX + 5 / + 1 / + 3
// columns. Cells outside the padded grid read as 0 and are never used by an existing face.
template <int DIR> struct TileShape {
    static constexpr int rows(int halo) { return DIR == 0 ? FBY + halo : FBY; }
    static constexpr int cols(int halo) { return DIR == 0 ? FBX : FBX + halo; }
    static constexpr int ncell = rows(5) * cols(5), nprep = rows(1) * cols(1), nsens = rows(3) * cols(3);
    static constexpr int total = 6 * ncell + 6 * nprep + 2 * nsens;
    static constexpr int sweep = DIR == 0 ? FBX : 1;  // tile stride along the sweep
};

template <int DIR, typename T> struct SmemView {
    const T *sm;
    int bc, bp, bs;  // this thread's cell 0 in the cell, first-order and sensor planes
    using S = TileShape<DIR>;
    __device__ __forceinline__ void cell(int o, T u[6]) const
    {
#pragma unroll
        for (int f = 0; f < 6; ++f) u[f] = sm[f * S::ncell + bc + o * S::sweep];
    }
    __device__ __forceinline__ T pr(int f, int o) const { return sm[6 * S::ncell + f * S::nprep + bp + o * S::sweep]; }
    __device__ __forceinline__ T un(int o) const { return pr(0, o); }
    __device__ __forceinline__ T ut(int o) const { return pr(1, o); }
    __device__ __forceinline__ T lp(int o) const { return pr(2, o); }
    __device__ __forceinline__ T la(int o) const { return pr(3, o); }
    __device__ __forceinline__ T lc(int o) const { return pr(4, o); }
    __device__ __forceinline__ T lE(int o) const { return pr(5, o); }
    __device__ __forceinline__ T sn(int f, int o) const
    {
        return sm[6 * S::ncell + 6 * S::nprep + f * S::nsens + bs + o * S::sweep];
    }
    __device__ __forceinline__ T sens_c(int o) const { return sn(0, o); }
    __device__ __forceinline__ T sens_s(int o) const { return sn(1, o); }
};

// Cooperative, coalesced copy of a (rows x cols) window of a padded-grid array starting at
// (row0, col0) into a shared-memory plane, by asynchronous global-to-shared copies (cp.async): every
// copy of the thread is in flight at once; the caller waits for all of them. Elements outside the
// array are zero-filled (source size 0, read from the plane's first element's address).
template <typename T>
__device__ __forceinline__ void stage(T *dst, const T *src, long long pitch, int row0, int col0, int rows, int cols,
                                      int nrow, int ncol, int tid)
{
    for (int k = tid; k < rows * cols; k += FBX * FBY) {
        const int r = k / cols, c = k - r * cols;
        const int gi = row0 + r, gj = col0 + c;
        const bool in = gi >= 0 && gi < nrow && gj >= 0 && gj < ncol;
        const T *from = in ? src + (long long)gi * pitch + gj : src;
        const unsigned to = (unsigned)__cvta_generic_to_shared(dst + k);
        if constexpr (sizeof(T) == 4)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(to), "l"(from), "r"(in ? 4 : 0)
                         : "memory");
        else
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(to), "l"(from), "r"(in ? 8 : 0)
                         : "memory");
    }
}

template <typename T> __device__ __forceinline__ const T *cell_plane(const Src32 &cs, int f)
{
    const float *a[6] = {cs.c.ar1, cs.c.ar2, cs.c.ru, cs.c.rv, cs.c.p, cs.c.al};
    return a[f];
}
template <typename T> __device__ __forceinline__ const T *cell_plane(const Src64 &cs, int f)
{
    const int idx[6] = {F_AR1, F_AR2, F_RU, F_RV, F_P, F_AL};
    return cs.q.f[idx[f]];
}

// The staged form of face_kernel: stage the block's tile, then compute its faces from it.
template <int DIR, int VAR, int REC, typename T, typename CS, typename FT>
__device__ __forceinline__ void staged_faces(const Grid &g, const Eos &e, const CS &cs, const PrepT<T> &p,
                                             const Face<FT> &hi, const Face<FT> &lo, int do_high, int do_low)
{
    using S = TileShape<DIR>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    const int tid = threadIdx.y * FBX + threadIdx.x;
    const int j0 = blockIdx.x * FBX + (DIR == 0 ? g.g : g.g - 1);
    const int i0 = blockIdx.y * FBY + (DIR == 0 ? g.g - 1 : g.g);
    // window origins of the three tiles (cells -2, 0 and -1 along the sweep)
    const int cr = DIR == 0 ? i0 - 2 : i0, cc = DIR == 0 ? j0 : j0 - 2;
    const int pr = i0, pc = j0;
    const int sr = DIR == 0 ? i0 - 1 : i0, sc = DIR == 0 ? j0 : j0 - 1;
    const long long cp = cs.pitch();
#pragma unroll
    for (int f = 0; f < 6; ++f)
        stage(sm + f * S::ncell, cell_plane<T>(cs, f), cp, cr, cc, S::rows(5), S::cols(5), g.nxg, g.nyg, tid);
    const T *prep[6] = {DIR == 0 ? p.lu : p.lv, DIR == 0 ? p.lv : p.lu, p.lp, p.la, p.lc, p.lE};
#pragma unroll
    for (int f = 0; f < 6; ++f)
        stage(sm + 6 * S::ncell + f * S::nprep, prep[f], g.nyg, pr, pc, S::rows(1), S::cols(1), g.nxg, g.nyg, tid);
    if (do_high) {
        T *sens = sm + 6 * S::ncell + 6 * S::nprep;
        stage(sens, DIR == 0 ? p.cx : p.cy, g.nyg, sr, sc, S::rows(3), S::cols(3), g.nxg, g.nyg, tid);
        if (VAR == kSC)
            stage(sens + S::nsens, DIR == 0 ? p.sx : p.sy, g.nyg, sr, sc, S::rows(3), S::cols(3), g.nxg, g.nyg, tid);
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    const int j = j0 + threadIdx.x, i = i0 + threadIdx.y;
    if (i >= g.g + g.nx || j >= g.g + g.ny) return;
    SmemView<DIR, T> v;
    v.sm = sm;
    const int ti = threadIdx.y, tj = threadIdx.x;
    if (DIR == 0) {
        v.bc = (ti + 2) * S::cols(5) + tj;
        v.bp = ti * S::cols(1) + tj;
        v.bs = (ti + 1) * S::cols(3) + tj;
    } else {
        v.bc = ti * S::cols(5) + tj + 2;
        v.bp = ti * S::cols(1) + tj;
        v.bs = ti * S::cols(3) + tj + 1;
    }
    face_body<DIR, VAR, REC, T, true>(e, v, hi, lo, do_high != 0, do_low != 0, (long long)i * g.nyg + j);
}

// Binary32 sweeps: registers capped for 8 resident blocks per SM (no spills; 64 registers instead
// of 89 lift the warp occupancy from 31 % to 50 % of the latency-bound kernel); binary64: kFace64Blocks.
// STAGED: the block's tile is staged in shared memory first (binary64: as fast as direct loads, the
// sweep being bound by the binary64 pipe); otherwise each face reads its stencil directly, through
// L1 (binary32: 55 ms against 89 ms staged per 10 steps of the triple point -- the staging's
// barrier serialises loads and compute within a block, and L1 already serves the reuse).
template <int DIR, int VAR, int REC, typename T, typename CS, typename FT, bool STAGED>
__global__ void __launch_bounds__(FBX *FBY, sizeof(T) == 4 ? 8 : kFace64Blocks)
face_kernel(Grid g, Eos e, CS cs, PrepT<T> p, Face<FT> hi, Face<FT> lo, int do_high, int do_low)
{
    if constexpr (!STAGED) {
        const int j = blockIdx.x * blockDim.x + threadIdx.x + (DIR == 0 ? g.g : g.g - 1);
        const int i = blockIdx.y * blockDim.y + threadIdx.y + (DIR == 0 ? g.g - 1 : g.g);
        if (i >= g.g + g.nx || j >= g.g + g.ny) return;
        face_body<DIR, VAR, REC, T, true>(e, GlobalView<DIR, T, CS>(g, cs, p, i, j), hi, lo, do_high != 0,
                                          do_low != 0, (long long)i * g.nyg + j);
    } else {
        staged_faces<DIR, VAR, REC, T>(g, e, cs, p, hi, lo, do_high, do_low);
    }
}

template <int DIR, int VAR, int REC, typename T, typename CS, typename FT>
void launch_one(const Grid &g, const Eos &e, const CS &cs, const PrepT<T> &p, const Face<FT> &hi,
                const Face<FT> &lo, bool high, bool low, cudaStream_t s)
{
    const int nj = DIR == 0 ? g.ny : g.ny + 1, ni = DIR == 0 ? g.nx + 1 : g.nx;
    dim3 grid((nj + FBX - 1) / FBX, (ni + FBY - 1) / FBY);
    constexpr bool staged = sizeof(T) == 8;
    const size_t bytes = staged ? sizeof(T) * TileShape<DIR>::total : 0;
    face_kernel<DIR, VAR, REC, T, CS, FT, staged><<<grid, dim3(FBX, FBY), bytes, s>>>(g, e, cs, p, hi, lo, high, low);
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
