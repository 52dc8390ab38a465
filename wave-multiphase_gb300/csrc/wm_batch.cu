// wm_batch.cu -- the batched form: many independent solves of uneven grid sizes advanced together
// by one persistent kernel launch (replayed from a captured CUDA graph), with the tile shape of
// every size class of grids chosen by a measuring autotuner.
//
// A batch has `capacity` slots; a slot holds one solve (its grid, equation of state, boundary
// rules, time limit and step budget, its caller-owned cell arrays and workspace) or is empty.
// wm_batch_run launches batch_kernel once: every block walks the batch's tile list through the
// phases of a stage (ghost fill x, ghost fill y, preparation, sensors, face sweeps, three limiter
// passes whose blends are rebuilt in registers, combine), separated by grid-wide barriers, three stages per step, then a
// per-solve time-step phase (dt from the solve's own CFL reduction, clamped to its end time), for
// up to `nsteps` steps. Solves that reach their end time or step budget drop out of later steps.
//
// Grid barriers spin on a generation counter with an iteration limit: a block that waits too long
// sets the batch's error flag, every block returns at the next barrier, and wm_batch_run reports
// WM_ERR_STATE. The kernel is launched cooperatively, which guarantees all its blocks are resident.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "../../include/wavemp.h"
#include "wm_bodies.cuh"

namespace wm {
void set_error_text(const char *msg);
}

using namespace wm;

namespace {

constexpr int kThreads = 128;
constexpr int kShapes = 4;
constexpr int kShapeTI[kShapes] = {1, 2, 4, 8};  // tile rows (x) x columns (y) = 128 cells
constexpr int kShapeTJ[kShapes] = {128, 64, 32, 16};
constexpr unsigned long long kSpinLimit = 1ull << 26;  // default wait limit (about 4 s of 64 ns naps)
constexpr int kPhaseSlots = 10;  // the 9 phases of a stage, then the end-of-step phase

struct SolveDev {
    Grid g;
    Eos e;
    int bc[4];
    Fields q, old;
    Face<double> fh, gh, fl, gl;
    Face<float> fh32, gh32, fl32, gl32;
    Prep prep;
    PrepT<float> prep32;
    Cells32 cells32;
    double *theta[3];
    float *theta32[3];
    unsigned long long *dt_bits;  // CFL reduction of the current step
    double *dt, *t;               // this step's dt, elapsed time
    long long *steps;
    int *done;
    double t_end;
    long long max_steps;
    double *dt_log;        // per-step dt record / replay buffer (caller-owned), or null
    long long dt_log_len;
    int dt_mode;           // 0 none, 1 record the dt of every step, 2 replay it
};

struct Tile {
    int slot;
    int i0, j0;
    int ti, tj;
};

struct BatchDev {
    SolveDev *solves;
    int nslots;
    const Tile *tiles;
    int ntiles;
    unsigned *bar_count, *bar_gen;
    int *err;
    const unsigned long long *spin_limit;  // waits a block may spin at a grid barrier before failing
    int repair;
    int sw64;                  // binary32 form: binary64 switches
    unsigned long long *prof;  // per-phase nanoseconds (block 0's view), or null
};

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ bool grid_barrier(const BatchDev &B)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = B.bar_gen;
        unsigned g0 = *gen;
        __threadfence();
        if (atomicAdd(B.bar_count, 1u) == gridDim.x - 1) {
            atomicExch(B.bar_count, 0u);
            __threadfence();
            atomicAdd(B.bar_gen, 1u);
        } else {
            const unsigned long long limit = *(volatile const unsigned long long *)B.spin_limit;
            unsigned long long spins = 0;
            while (*gen == g0) {
                if (++spins > limit) {
                    atomicExch(B.err, 1);
                    break;
                }
                if (*(volatile int *)B.err) break;
                __nanosleep(64);
            }
        }
    }
    __syncthreads();
    __threadfence();  // every thread: later loads must not see lines this SM cached before the barrier
    return *(volatile int *)B.err == 0;
}

// Ghost fill of one cell, x pass (bc_x_kernel, SC:1616-1646, per side rule); `save` copies the
// pre-fill value to the step-start state first (copy_old precedes apply_bc, SC:2033-2036).
__device__ __forceinline__ void bcx_cell(const SolveDev &S, bool save, int i, int j)
{
    const Grid &g = S.g;
    if (j >= g.nyg || i >= g.nxg) return;
    int src, side;
    if (i < g.g) {
        src = g.g;
        side = 0;
    } else if (i >= g.g + g.nx) {
        src = g.g + g.nx - 1;
        side = 1;
    } else {
        return;
    }
    const long long k = kf_of(S.q, i, j), ks = kf_of(S.q, src, j);
#pragma unroll
    for (int c = 0; c < 9; ++c) {
        double *a = S.q.f[c];
        if (save && c < 6) S.old.f[c][(long long)i * S.old.pitch + j] = a[k];
        double v = a[ks];
        if ((c == F_RU || c == F_U) && S.bc[side] == 1) v = -1.0 * v;
        a[k] = v;
    }
}

// y pass (bc_y_kernel, SC:1650-1682); corners take the y rule; corners were saved by the x pass.
__device__ __forceinline__ void bcy_cell(const SolveDev &S, bool save, int i, int j)
{
    const Grid &g = S.g;
    if (j >= g.nyg || i >= g.nxg) return;
    int src, side;
    if (j < g.g) {
        src = g.g;
        side = 2;
    } else if (j >= g.g + g.ny) {
        src = g.g + g.ny - 1;
        side = 3;
    } else {
        return;
    }
    const bool save_here = save && i >= g.g && i < g.g + g.nx;
    const long long k = kf_of(S.q, i, j), ks = kf_of(S.q, i, src);
#pragma unroll
    for (int c = 0; c < 9; ++c) {
        double *a = S.q.f[c];
        if (save_here && c < 6) S.old.f[c][(long long)i * S.old.pitch + j] = a[k];
        double v = a[ks];
        if ((c == F_RV || c == F_V) && S.bc[side] == 1) v = -1.0 * v;
        a[k] = v;
    }
}

// The limiter's blends are rebuilt in registers by the next pass and by the combine (CellFaces),
// so a stage has no blend phases.
enum Phase { PH_BCX, PH_BCY, PH_PREP, PH_SENSOR, PH_FACES, PH_THETA0, PH_THETA1, PH_THETA2, PH_FINAL,
             PH_BLEND0, PH_BLEND1, PH_BLEND2 };
// The phases of a stage. Binary32: the limiter passes rebuild the earlier passes' blends in
// registers and the combine all three (no blend phases: binary32 blends are cheap, the traffic is
// what counts). Binary64: each pass is followed by the in-place blend of pp_blend_*_flux_kernel
// (SC:1479-1548), so the passes and the combine read the blended fluxes as they are -- the
// per-solve path's form, whose binary64 blend arithmetic is done once per face instead of again in
// every later pass and in the combine.
constexpr int kPhases32 = 9, kPhases64 = 12;
template <int FP32> __device__ __forceinline__ int phase_at(int k)
{
    if (FP32 || k < 6) return k;  // BCX .. THETA0, then (binary32) THETA1, THETA2, FINAL
    switch (k) {
    case 6: return PH_BLEND0;
    case 7: return PH_THETA1;
    case 8: return PH_BLEND1;
    case 9: return PH_THETA2;
    case 10: return PH_BLEND2;
    default: return PH_FINAL;
    }
}
// profile slot of a phase: a blend's time counts with its limiter pass
__device__ __forceinline__ int prof_slot(int ph) { return ph >= PH_BLEND0 ? PH_THETA0 + (ph - PH_BLEND0) : ph; }

template <int VAR, int REC, int FP32>
__device__ __forceinline__ void run_phase(const BatchDev &B, int phase, int stage)
{
    const double alpha = stage == 0 ? 0.0 : (stage == 1 ? 0.75 : 1.0 / 3.0);
    const double beta = stage == 0 ? 1.0 : (stage == 1 ? 0.25 : 2.0 / 3.0);
    const int tid = threadIdx.x;
    // the face phase sweeps the tile list twice, x faces then y faces (no barrier between them:
    // they share no data), so that a block runs one face body at a time
    const int passes = phase == PH_FACES ? 2 : 1;
    for (int pass = 0; pass < passes; ++pass)
    for (int t = blockIdx.x; t < B.ntiles; t += gridDim.x) {
        const Tile tl = B.tiles[t];
        const SolveDev &S = B.solves[tl.slot];
        if (*(volatile int *)S.done) continue;  // uniform per tile
        const Grid &g = S.g;
        const int i = tl.i0 + tid / tl.tj, j = tl.j0 + tid % tl.tj;
        const bool in = i < g.nxg && j < g.nyg;
        const bool interior = in && i >= g.g && i < g.g + g.nx && j >= g.g && j < g.g + g.ny;
        const double dt = *S.dt;
        switch (phase) {
        case PH_BCX:
            bcx_cell(S, stage == 0, i, j);
            break;
        case PH_BCY:
            bcy_cell(S, stage == 0, i, j);
            break;
        case PH_PREP:
            if (in) {
                if (FP32)
                    prep32_body(g, S.e, S.q, S.prep32, S.cells32, B.sw64 != 0, true, i, j);
                else
                    prep_body(g, S.e, S.q, S.prep, true, i, j);
            }
            break;
        case PH_SENSOR:
            if (in) {
                if (FP32)
                    sensor32_body(g, S.e, S.q, S.prep32, S.cells32, VAR == kSC, B.sw64 != 0, true, i, j);
                else
                    sensor_body(g, S.e, S.q, S.prep, VAR == kSC, true, i, j);
            }
            break;
        case PH_FACES: {
            const bool xf = pass == 0 && i >= g.g - 1 && i < g.g + g.nx && j >= g.g && j < g.g + g.ny;
            const bool yf = pass == 1 && i >= g.g && i < g.g + g.nx && j >= g.g - 1 && j < g.g + g.ny;
            const long long kw = kw_of(g, i, j);
            if (FP32) {
                const Src32 cs{S.cells32, g.nyg};
                if (xf) face_body<0, VAR, REC, float>(S.e, GlobalView<0, float, Src32>(g, cs, S.prep32, i, j), S.fh32, S.fl32, true, true, kw);
                if (yf) face_body<1, VAR, REC, float>(S.e, GlobalView<1, float, Src32>(g, cs, S.prep32, i, j), S.gh32, S.gl32, true, true, kw);
            } else {
                const Src64 cs{S.q};
                if (xf) face_body<0, VAR, REC, double>(S.e, GlobalView<0, double, Src64>(g, cs, S.prep, i, j), S.fh, S.fl, true, true, kw);
                if (yf) face_body<1, VAR, REC, double>(S.e, GlobalView<1, double, Src64>(g, cs, S.prep, i, j), S.gh, S.gl, true, true, kw);
            }
            break;
        }
        case PH_THETA0:
        case PH_THETA1:
        case PH_THETA2:
            if (interior) {
                double th;
                const int p = phase - PH_THETA0;
                if (FP32) {
                    const Cells32 &c = S.cells32;
                    th = p == 0 ? theta_body<0, float, 0>(g, S.e, S.q, c, S.fh32, S.gh32, S.fl32, S.gl32, dt, S.theta32, i, j)
                       : p == 1 ? theta_body<1, float, 1>(g, S.e, S.q, c, S.fh32, S.gh32, S.fl32, S.gl32, dt, S.theta32, i, j)
                                : theta_body<2, float, 2>(g, S.e, S.q, c, S.fh32, S.gh32, S.fl32, S.gl32, dt, S.theta32, i, j);
                    S.theta32[p][kw_of(g, i, j)] = store_as<float>(th);
                } else {  // the earlier passes' blends are in place
                    const Cells32 none32{};
                    th = p == 0 ? theta_body<0, double, 0>(g, S.e, S.q, none32, S.fh, S.gh, S.fl, S.gl, dt, S.theta, i, j)
                       : p == 1 ? theta_body<1, double, 0>(g, S.e, S.q, none32, S.fh, S.gh, S.fl, S.gl, dt, S.theta, i, j)
                                : theta_body<2, double, 0>(g, S.e, S.q, none32, S.fh, S.gh, S.fl, S.gl, dt, S.theta, i, j);
                    S.theta[p][kw_of(g, i, j)] = th;
                }
            }
            break;
        case PH_BLEND0:
        case PH_BLEND1:
        case PH_BLEND2:  // binary64 only: the faces of cells g-1 .. g+n-1 (blend_kernel's range)
            if (!FP32 && i >= g.g - 1 && i < g.g + g.nx && j >= g.g - 1 && j < g.g + g.ny)
                blend_body<double>(g, S.fh, S.gh, S.fl, S.gl, S.theta[phase - PH_BLEND0], i, j);
            break;
        case PH_FINAL: {
            unsigned flags = FIN_RK3 | FIN_PRIM;
            if (B.repair) flags |= FIN_ADMISSIBLE;
            if (stage != 0) flags |= FIN_OLD_READ;
            if (stage == 0) flags |= FIN_SAVE_OLD;
            if (stage == 2) flags |= FIN_DT;
            const Counters none = {nullptr, nullptr, nullptr, nullptr};
            unsigned long long bits;
            if (FP32)
                bits = final_body<float, 3>(g, S.e, flags, S.q, S.old, S.fh32, S.gh32, S.fl32, S.gl32, S.theta32,
                                            dt, nullptr, alpha, beta, none, i, j);
            else
                bits = final_body<double, 0>(g, S.e, flags, S.q, S.old, S.fh, S.gh, S.fl, S.gl, S.theta, dt,
                                             nullptr, alpha, beta, none, i, j);
            if (stage == 2) {  // every lane of the warp takes part (tiles are warp multiples)
                for (int o = 16; o > 0; o >>= 1) {
                    unsigned long long other = __shfl_down_sync(0xffffffffu, bits, o);
                    bits = other < bits ? other : bits;
                }
                if ((tid & 31) == 0 && bits != ~0ull) atomicMin(S.dt_bits, bits);
            }
            break;
        }
        }
    }
}

// Resident blocks per SM the persistent kernel is compiled for (its phases share one register
// allocation, so every phase runs at this occupancy). Binary32 form: 8 (64 registers, a few dozen
// bytes of spills in the face phase, more warps for the memory- and binary64-bound phases).
// Binary64 form: 4 (128 registers, under 300 bytes of spills in the face phase). Measured on the 64
// config-3 droplets with the in-place blend phases: 203 / 249 / 264 Mcell-stage/s at 2 (uncapped,
// 196 registers) / 3 / 4 blocks, against 235 for the same solves run one after another.
constexpr int kMinBlocksFp32 = 8;
#ifndef WM_BATCH64_MIN_BLOCKS
#define WM_BATCH64_MIN_BLOCKS 4
#endif
constexpr int kMinBlocksFp64 = WM_BATCH64_MIN_BLOCKS;

template <int VAR, int REC, int FP32>
__global__ void __launch_bounds__(kThreads, FP32 ? kMinBlocksFp32 : kMinBlocksFp64) batch_kernel(BatchDev B, int nsteps)
{
    // Phase timing: a phase ends when the grid barrier after it opens, so block 0's clock between
    // successive barrier exits is the phase's duration across the whole grid.
    const bool timing = B.prof != nullptr && blockIdx.x == 0 && threadIdx.x == 0;
    unsigned long long last = timing ? global_ns() : 0;
    for (int step = 0; step < nsteps; ++step) {
        for (int stage = 0; stage < 3; ++stage) {
#pragma unroll 1
            for (int k = 0; k < (FP32 ? kPhases32 : kPhases64); ++k) {
                const int ph = phase_at<FP32>(k);
                run_phase<VAR, REC, FP32>(B, ph, stage);
                if (!grid_barrier(B)) return;
                if (timing) {
                    const unsigned long long now = global_ns();
                    B.prof[prof_slot(ph)] += now - last;
                    last = now;
                }
            }
        }
        // End of the step: the next dt of every unfinished solve from its own CFL reduction
        // (timestep_kernel + get_dt, SC:1686-1705), its time and step count, the end-time clamp of
        // the reference's time loop (SC:2021-2026, without the save times) and the stop test.
        if (blockIdx.x == 0) {
            for (int s = threadIdx.x; s < B.nslots; s += blockDim.x) {
                SolveDev &S = B.solves[s];
                if (!S.done || *S.done) continue;
                double dt_next = S.g.cfl * __longlong_as_double((long long)*S.dt_bits);
                *S.dt_bits = (unsigned long long)__double_as_longlong(1.0e30);
                double t = *S.t + *S.dt;
                *S.t = t;
                long long n = *S.steps + 1;
                *S.steps = n;
                if (S.dt_mode == 1 && n - 1 < S.dt_log_len) S.dt_log[n - 1] = *S.dt;
                if (S.dt_mode == 2 && n < S.dt_log_len) dt_next = S.dt_log[n];
                bool stop = (S.max_steps > 0 && n >= S.max_steps) || !(dt_next > 0.0);
                if (S.t_end > 0.0) {
                    if (t >= S.t_end - 1.0e-14 * S.t_end)
                        stop = true;
                    else if (t + dt_next > S.t_end)
                        dt_next = S.t_end - t;
                }
                *S.dt = dt_next;
                if (stop) *S.done = 1;
            }
        }
        if (!grid_barrier(B)) return;
        if (timing) {
            const unsigned long long now = global_ns();
            B.prof[kPhaseSlots - 1] += now - last;
            last = now;
        }
    }
}

// Initial dt of one slot from its current state (get_dt, SC:1986-1995), clamped to its end time.
__global__ void batch_init_dt_kernel(SolveDev *solves, int slot)
{
    SolveDev &S = solves[slot];
    double dt = S.g.cfl * __longlong_as_double((long long)*S.dt_bits);
    *S.dt_bits = (unsigned long long)__double_as_longlong(1.0e30);
    if (S.dt_mode == 2 && S.dt_log_len > 0) dt = S.dt_log[0];
    if (S.t_end > 0.0 && *S.t + dt > S.t_end) dt = S.t_end - *S.t;
    *S.dt = dt;
}

using KernelFn = void (*)(BatchDev, int);

KernelFn pick_kernel(int variant, int recon, int precision)
{
    const bool f = precision == WM_PREC_FP32;
    if (variant == WM_VARIANT_SC && recon == WM_RECON_SHIPPED) return f ? batch_kernel<kSC, kMuscl, 1> : batch_kernel<kSC, kMuscl, 0>;
    if (variant == WM_VARIANT_SC && recon == WM_RECON_MP5C6) return f ? batch_kernel<kSC, kMp5, 1> : batch_kernel<kSC, kMp5, 0>;
    if (variant == WM_VARIANT_M10 && recon == WM_RECON_SHIPPED) return f ? batch_kernel<kM10, kMuscl, 1> : batch_kernel<kM10, kMuscl, 0>;
    return f ? batch_kernel<kM10, kMp5, 1> : batch_kernel<kM10, kMp5, 0>;
}

constexpr size_t kAlign = 256;
size_t arr_bytes(int nx, int ny, int g, size_t elem)
{
    size_t n = (size_t)(nx + 2 * g) * (size_t)(ny + 2 * g) * elem;
    return (n + kAlign - 1) / kAlign * kAlign;
}

int size_class(long long cells)
{
    int c = 0;
    while ((1ll << (c + 1)) <= cells && c < 40) ++c;
    return c;  // floor(log2(cells))
}

void set_err(const char *where, cudaError_t e)
{
    char msg[256];
    snprintf(msg, sizeof msg, "%s: %s", where, cudaGetErrorString(e));
    set_error_text(msg);
}

}  // namespace

struct wm_batch {
    wm_batch_params P;
    int capacity;
    std::vector<SolveDev> host;  // host copies of the slot descriptors
    std::vector<char> used;
    SolveDev *d_solves = nullptr;
    void *d_small = nullptr;  // per-slot scalars + barrier + error flag
    Tile *d_tiles = nullptr;
    size_t tile_cap = 0;
    int ntiles = 0;
    bool dirty = true;
    std::map<int, int> shape_of_class;  // size class -> tile shape index
    int fixed_shape = -1;
    int grid = 0;
    KernelFn fn = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_steps = 0;
    bool graph_ok = true;
    unsigned *bar_count = nullptr, *bar_gen = nullptr;
    int *err = nullptr;
    unsigned long long *spin_limit = nullptr;  // in d_small's tail
    unsigned long long *prof = nullptr;  // kPhaseSlots counters in d_small's tail
    bool prof_on = false;
};

namespace {

// Per-slot scalars in d_small: dt_bits, dt, t, steps, done (8 bytes each), then the barrier words.
constexpr size_t kSlotScalars = 5;

void slot_scalars(wm_batch *b, int s, SolveDev &S)
{
    char *base = static_cast<char *>(b->d_small) + (size_t)s * kSlotScalars * 8;
    S.dt_bits = reinterpret_cast<unsigned long long *>(base);
    S.dt = reinterpret_cast<double *>(base + 8);
    S.t = reinterpret_cast<double *>(base + 16);
    S.steps = reinterpret_cast<long long *>(base + 24);
    S.done = reinterpret_cast<int *>(base + 32);
}

int rebuild_tiles(wm_batch *b)
{
    std::vector<Tile> tiles;
    for (int s = 0; s < b->capacity; ++s) {
        if (!b->used[s]) continue;
        const Grid &g = b->host[s].g;
        long long cells = (long long)g.nx * g.ny;
        int sh = b->fixed_shape >= 0 ? b->fixed_shape : 2;
        auto it = b->shape_of_class.find(size_class(cells));
        if (b->fixed_shape < 0 && it != b->shape_of_class.end()) sh = it->second;
        const int ti = kShapeTI[sh], tj = kShapeTJ[sh];
        for (int i0 = 0; i0 < g.nxg; i0 += ti)
            for (int j0 = 0; j0 < g.nyg; j0 += tj) tiles.push_back({s, i0, j0, ti, tj});
    }
    // interleave slots so that consecutive tiles (one per block) come from different solves
    std::stable_sort(tiles.begin(), tiles.end(), [](const Tile &a, const Tile &c) { return a.i0 < c.i0; });
    b->ntiles = (int)tiles.size();
    if ((size_t)b->ntiles > b->tile_cap) {
        if (b->d_tiles) cudaFree(b->d_tiles);
        b->tile_cap = std::max<size_t>((size_t)b->ntiles, 1024);
        cudaError_t e = cudaMalloc(&b->d_tiles, b->tile_cap * sizeof(Tile));
        if (e != cudaSuccess) {
            b->d_tiles = nullptr;
            b->tile_cap = 0;
            set_err("wm_batch tiles", e);
            return WM_ERR_NOMEM;
        }
    }
    if (b->ntiles) {
        cudaError_t e = cudaMemcpy(b->d_tiles, tiles.data(), tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            set_err("wm_batch tiles", e);
            return WM_ERR_CUDA;
        }
    }
    cudaError_t e = cudaMemcpy(b->d_solves, b->host.data(), b->capacity * sizeof(SolveDev), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_err("wm_batch solves", e);
        return WM_ERR_CUDA;
    }
    b->dirty = false;
    if (b->graph_exec) {
        cudaGraphExecDestroy(b->graph_exec);
        b->graph_exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    return WM_OK;
}

int launch(wm_batch *b, int nsteps, cudaStream_t s)
{
    BatchDev B;
    B.solves = b->d_solves;
    B.nslots = b->capacity;
    B.tiles = b->d_tiles;
    B.ntiles = b->ntiles;
    B.bar_count = b->bar_count;
    B.bar_gen = b->bar_gen;
    B.err = b->err;
    B.spin_limit = b->spin_limit;
    B.repair = b->P.emergency_repair;
    B.sw64 = b->P.fp64_switches;
    B.prof = b->prof_on ? b->prof : nullptr;
    void *args[] = {&B, &nsteps};
    int grid = std::max(1, std::min(b->grid, b->ntiles));
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)b->fn, dim3(grid), dim3(kThreads), args, 0, s);
    if (e != cudaSuccess) {
        set_err("wm_batch_run launch", e);
        return WM_ERR_CUDA;
    }
    return WM_OK;
}

}  // namespace

extern "C" {

size_t wm_solve_workspace_bytes(const wm_batch_params *p, int nx, int ny)
{
    if (!p || nx < 1 || ny < 1) return 0;
    const int g = p->g;
    const size_t fin = 2 * arr_bytes(nx, ny, g, 1);  // first-order finiteness bytes, x and y
    // the switch pre-check's pairs: 3 binary32 arrays (precision form) or 4 beyond the density pair
    if (p->precision == WM_PREC_FP32)
        return (size_t)(28 + 3 + 11 + 9 + 3) * arr_bytes(nx, ny, g, 4) + arr_bytes(nx, ny, g, 8) + fin;
    return (size_t)42 * arr_bytes(nx, ny, g, 8) + (size_t)(1 + 4) * arr_bytes(nx, ny, g, 4) + fin;
}

int wm_batch_create(const wm_batch_params *p, int capacity, wm_batch **out)
{
    if (!out) return WM_ERR_INVALID;
    *out = nullptr;
    if (!p || capacity < 1 || capacity > (1 << 20) || p->g < 4 || p->g > 64 || !(p->cfl > 0.0)) return WM_ERR_INVALID;
    if (p->variant != WM_VARIANT_SC && p->variant != WM_VARIANT_M10) return WM_ERR_INVALID;
    if (p->recon != WM_RECON_SHIPPED && p->recon != WM_RECON_MP5C6) return WM_ERR_INVALID;
    if (p->precision != WM_PREC_FP64 && p->precision != WM_PREC_FP32) return WM_ERR_INVALID;
    if (p->tile_shape < -1 || p->tile_shape >= kShapes) return WM_ERR_INVALID;
    wm_batch *b = new (std::nothrow) wm_batch();
    if (!b) return WM_ERR_NOMEM;
    b->P = *p;
    b->capacity = capacity;
    b->fixed_shape = p->tile_shape;
    b->host.assign(capacity, SolveDev{});
    b->used.assign(capacity, 0);
    size_t small = (size_t)capacity * kSlotScalars * 8 + 256;
    cudaError_t e = cudaMalloc(&b->d_small, small);
    if (e == cudaSuccess) e = cudaMemset(b->d_small, 0, small);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_solves, capacity * sizeof(SolveDev));
    if (e != cudaSuccess) {
        set_err("wm_batch_create", e);
        cudaFree(b->d_small);
        cudaFree(b->d_solves);
        delete b;
        return WM_ERR_NOMEM;
    }
    char *tail = static_cast<char *>(b->d_small) + (size_t)capacity * kSlotScalars * 8;
    b->bar_count = reinterpret_cast<unsigned *>(tail);
    b->bar_gen = reinterpret_cast<unsigned *>(tail + 4);
    b->err = reinterpret_cast<int *>(tail + 8);
    b->spin_limit = reinterpret_cast<unsigned long long *>(tail + 16);
    b->prof = reinterpret_cast<unsigned long long *>(tail + 64);  // kPhaseSlots x 8 bytes, within the 256
    {
        const unsigned long long limit = p->spin_limit > 0 ? (unsigned long long)p->spin_limit : kSpinLimit;
        e = cudaMemcpy(b->spin_limit, &limit, sizeof limit, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            set_err("wm_batch_create", e);
            cudaFree(b->d_small);
            cudaFree(b->d_solves);
            delete b;
            return WM_ERR_CUDA;
        }
    }
    for (int s = 0; s < capacity; ++s) {
        slot_scalars(b, s, b->host[s]);
        b->host[s].done = nullptr;  // empty slot: no done flag, skipped by the kernel's step end
    }
    b->fn = pick_kernel(p->variant, p->recon, p->precision);
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)b->fn, kThreads, 0);
    b->grid = std::max(1, per_sm) * sms;
    *out = b;
    return WM_OK;
}

void wm_batch_destroy(wm_batch *b)
{
    if (!b) return;
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    cudaFree(b->d_tiles);
    cudaFree(b->d_solves);
    cudaFree(b->d_small);
    delete b;
}

int wm_batch_set(wm_batch *b, int slot, const wm_solve_desc *d, void *workspace, size_t bytes)
{
    if (!b || !d || slot < 0 || slot >= b->capacity || !workspace) return WM_ERR_INVALID;
    const int g = b->P.g;
    if (d->nx < 1 || d->ny < 1 || !(d->dx > 0.0) || !(d->dy > 0.0) || !(d->gamma1 > 1.0) || !(d->gamma2 > 1.0))
        return WM_ERR_INVALID;
    for (int k = 0; k < 4; ++k)
        if (d->bc[k] != WM_BC_TRANSMISSIVE && d->bc[k] != WM_BC_SLIP) return WM_ERR_INVALID;
    const int nyg = d->ny + 2 * g;
    const wm_fields *fs[2] = {&d->q, &d->q_old};
    for (int w = 0; w < 2; ++w) {
        const wm_fields *f = fs[w];
        if (f->pitch < nyg) return WM_ERR_INVALID;
        double *const ptr[10] = {f->ar1, f->ar2, f->ru, f->rv, f->E, f->al, f->u_p, f->v_p, f->p_p, f->al_prim};
        for (int c = 0; c < (w == 0 ? 10 : 6); ++c)
            if (!ptr[c]) return WM_ERR_INVALID;
    }
    if (bytes < wm_solve_workspace_bytes(&b->P, d->nx, d->ny) || ((uintptr_t)workspace % kAlign)) return WM_ERR_NOMEM;

    SolveDev &S = b->host[slot];
    Grid &G = S.g;
    G.nx = d->nx; G.ny = d->ny; G.g = g; G.nxg = d->nx + 2 * g; G.nyg = nyg; G.pitch = nyg;
    G.dx = d->dx; G.dy = d->dy; G.inv_dx = 1.0 / d->dx; G.inv_dy = 1.0 / d->dy; G.inv_dxf = float(G.inv_dx); G.inv_dyf = float(G.inv_dy); G.cfl = b->P.cfl;
    S.e = make_eos(d->gamma1, d->pinf1, d->gamma2, d->pinf2);
    for (int k = 0; k < 4; ++k) S.bc[k] = d->bc[k];
    Fields *dst[2] = {&S.q, &S.old};
    for (int w = 0; w < 2; ++w) {
        const wm_fields *f = fs[w];
        Fields &F = *dst[w];
        F.f[0] = f->ar1; F.f[1] = f->ar2; F.f[2] = f->ru; F.f[3] = f->rv; F.f[4] = f->E; F.f[5] = f->al;
        F.f[6] = f->u_p; F.f[7] = f->v_p; F.f[8] = f->p_p; F.f[9] = f->al_prim;
        F.pitch = f->pitch;
    }
    S.t_end = d->t_end;
    S.max_steps = d->max_steps;
    S.dt_log = nullptr;  // no dt record / replay until wm_batch_dt_log
    S.dt_log_len = 0;
    S.dt_mode = 0;
    char *cur = static_cast<char *>(workspace);
    const size_t cells = (size_t)(d->nx + 2 * g) * (size_t)(d->ny + 2 * g);
    if (b->P.precision == WM_PREC_FP32) {
        size_t a4 = arr_bytes(d->nx, d->ny, g, 4);
        float *f4[28 + 11 + 9 + 3];
        for (int a = 0; a < 28 + 11 + 9 + 3; ++a) {
            f4[a] = reinterpret_cast<float *>(cur);
            cur += a4;
        }
        for (int c = 0; c < 7; ++c) {
            S.fh32.f[c] = f4[c]; S.gh32.f[c] = f4[7 + c]; S.fl32.f[c] = f4[14 + c]; S.gl32.f[c] = f4[21 + c];
        }
        PrepT<float> &P = S.prep32;
        P.sx = f4[28]; P.sy = f4[29]; P.ent = f4[30]; P.cx = f4[31]; P.cy = f4[32]; P.lu = f4[33];
        P.lv = f4[34]; P.lp = f4[35]; P.la = f4[36]; P.lc = f4[37]; P.lE = f4[38];
        Cells32 &C = S.cells32;
        C.ar1 = f4[39]; C.ar2 = f4[40]; C.ru = f4[41]; C.rv = f4[42]; C.p = f4[43]; C.al = f4[44];
        C.u = f4[45]; C.v = f4[46]; C.E = f4[47];
        for (int k = 0; k < 3; ++k) S.theta32[k] = f4[48 + k];
        P.ent64 = reinterpret_cast<double *>(cur);
        P.ent32 = P.ent;
        cur += arr_bytes(d->nx, d->ny, g, 8);
        set_pairs(P.pair, reinterpret_cast<float *>(P.ent64), cells, cur, a4, C.p);
        cur += 3 * a4;
        S.fl32.fin = reinterpret_cast<unsigned char *>(cur);
        S.gl32.fin = S.fl32.fin + arr_bytes(d->nx, d->ny, g, 1);
    } else {
        size_t a8 = arr_bytes(d->nx, d->ny, g, 8);
        double *f8[42];
        for (int a = 0; a < 42; ++a) {
            f8[a] = reinterpret_cast<double *>(cur);
            cur += a8;
        }
        for (int c = 0; c < 7; ++c) {
            S.fh.f[c] = f8[c]; S.gh.f[c] = f8[7 + c]; S.fl.f[c] = f8[14 + c]; S.gl.f[c] = f8[21 + c];
        }
        for (int k = 0; k < 3; ++k) S.theta[k] = f8[28 + k];
        Prep &P = S.prep;
        P.sx = f8[31]; P.sy = f8[32]; P.ent = f8[33]; P.cx = f8[34]; P.cy = f8[35]; P.lu = f8[36];
        P.lv = f8[37]; P.lp = f8[38]; P.la = f8[39]; P.lc = f8[40]; P.lE = f8[41];
        P.ent64 = f8[33];
        P.ent32 = reinterpret_cast<float *>(cur);  // the binary32 entropy of the switch pre-check
        const size_t a4 = arr_bytes(d->nx, d->ny, g, 4);
        cur += a4;
        set_pairs(P.pair, reinterpret_cast<float *>(f8[33]), cells, cur, a4, nullptr);
        cur += 4 * a4;
        S.fl.fin = reinterpret_cast<unsigned char *>(cur);
        S.gl.fin = S.fl.fin + arr_bytes(d->nx, d->ny, g, 1);
    }
    slot_scalars(b, slot, S);
    // zero the slot's scalars (t, steps, done) and set the CFL accumulator to get_dt's start value
    unsigned long long init[kSlotScalars] = {(unsigned long long)0x46293e5939a08ceaull, 0, 0, 0, 0};
    cudaError_t e = cudaMemcpy(S.dt_bits, init, sizeof init, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_err("wm_batch_set", e);
        return WM_ERR_CUDA;
    }
    b->used[slot] = 1;
    b->dirty = true;
    return WM_OK;
}

int wm_batch_clear(wm_batch *b, int slot)
{
    if (!b || slot < 0 || slot >= b->capacity) return WM_ERR_INVALID;
    b->used[slot] = 0;
    b->host[slot] = SolveDev{};
    slot_scalars(b, slot, b->host[slot]);
    b->host[slot].done = nullptr;
    b->dirty = true;
    return WM_OK;
}

int wm_batch_init_dt(wm_batch *b, int slot, void *stream)
{
    if (!b || slot < 0 || slot >= b->capacity || !b->used[slot]) return WM_ERR_INVALID;
    if (b->dirty) {
        int rc = rebuild_tiles(b);
        if (rc) return rc;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const SolveDev &S = b->host[slot];
    Counters c = {nullptr, nullptr, nullptr, S.dt_bits};
    launch_dt_reset(c, s);
    launch_dt_cell(S.g, S.e, S.q, c, s);
    batch_init_dt_kernel<<<1, 1, 0, s>>>(b->d_solves, slot);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_err("wm_batch_init_dt", e);
        return WM_ERR_CUDA;
    }
    return WM_OK;
}

int wm_batch_run(wm_batch *b, int nsteps, void *stream)
{
    if (!b || nsteps < 1) return WM_ERR_INVALID;
    if (b->dirty) {
        int rc = rebuild_tiles(b);
        if (rc) return rc;
    }
    if (b->ntiles == 0) return WM_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (b->graph_ok && (!b->graph_exec || b->graph_steps != nsteps)) {
        if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->graph_exec = nullptr;
        b->graph = nullptr;
        cudaStream_t cap;
        e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
        if (e == cudaSuccess) {
            e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
            int rc = e == cudaSuccess ? launch(b, nsteps, cap) : WM_ERR_CUDA;
            cudaGraph_t gr = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(cap, &gr);
            if (rc == WM_OK && e2 == cudaSuccess && gr &&
                cudaGraphInstantiate(&b->graph_exec, gr, 0) == cudaSuccess) {
                b->graph = gr;
                b->graph_steps = nsteps;
            } else {
                if (gr) cudaGraphDestroy(gr);
                b->graph_exec = nullptr;
                b->graph_ok = false;  // fall back to direct cooperative launches
            }
            cudaStreamDestroy(cap);
        } else {
            b->graph_ok = false;
        }
        cudaGetLastError();
    }
    if (b->graph_exec) {
        e = cudaGraphLaunch(b->graph_exec, s);
        if (e != cudaSuccess) {
            set_err("wm_batch_run graph", e);
            return WM_ERR_CUDA;
        }
        return WM_OK;
    }
    return launch(b, nsteps, s);
}

int wm_batch_query(wm_batch *b, wm_solve_status *out, void *stream)
{
    if (!b || !out) return WM_ERR_INVALID;
    std::vector<unsigned long long> raw((size_t)b->capacity * kSlotScalars + 2);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(raw.data(), b->d_small, raw.size() * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_err("wm_batch_query", e);
        return WM_ERR_CUDA;
    }
    for (int k = 0; k < b->capacity; ++k) {
        const unsigned long long *r = raw.data() + (size_t)k * kSlotScalars;
        double dt, t;
        long long steps;
        memcpy(&dt, r + 1, 8);
        memcpy(&t, r + 2, 8);
        memcpy(&steps, r + 3, 8);
        out[k].used = b->used[k];
        out[k].dt = dt;
        out[k].t = t;
        out[k].steps = steps;
        out[k].done = b->used[k] ? (int)(r[4] & 0xffffffffu) : 1;
    }
    int errflag = (int)(raw[(size_t)b->capacity * kSlotScalars + 1] & 0xffffffffu);
    if (errflag) {
        // Report once, then clear the flag and the barrier counters (blocks that gave up left the
        // arrival count part-way), so that the batch runs again once the caller has put its solves
        // back in a known state: a run that timed out stopped its solves part-way through a phase.
        e = cudaMemsetAsync(b->bar_count, 0, 12, s);  // count, generation, error flag
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        set_error_text(e == cudaSuccess
                           ? "wm_batch: a grid barrier timed out; the solves stopped part-way (flag cleared)"
                           : "wm_batch: a grid barrier timed out and the flag could not be cleared");
        return WM_ERR_STATE;
    }
    return WM_OK;
}

int wm_batch_tile_shape(wm_batch *b, int size_class_, int shape)
{
    if (!b || shape < 0 || shape >= kShapes || size_class_ < 0) return WM_ERR_INVALID;
    b->shape_of_class[size_class_] = shape;
    b->dirty = true;
    return WM_OK;
}

int wm_batch_spin_limit(wm_batch *b, long long limit)
{
    if (!b) return WM_ERR_INVALID;
    const unsigned long long v = limit > 0 ? (unsigned long long)limit : kSpinLimit;
    cudaError_t e = cudaMemcpy(b->spin_limit, &v, sizeof v, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_err("wm_batch_spin_limit", e);
        return WM_ERR_CUDA;
    }
    return WM_OK;
}

int wm_batch_scalars(wm_batch *b, void *host, int write, void *stream)
{
    if (!b || !host) return WM_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t n = (size_t)b->capacity * kSlotScalars * 8;
    cudaError_t e = write ? cudaMemcpyAsync(b->d_small, host, n, cudaMemcpyHostToDevice, s)
                          : cudaMemcpyAsync(host, b->d_small, n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_err("wm_batch_scalars", e);
        return WM_ERR_CUDA;
    }
    return WM_OK;
}

int wm_batch_dt_log(wm_batch *b, int slot, double *log, long long len, int mode)
{
    if (!b || slot < 0 || slot >= b->capacity || !b->used[slot] || mode < 0 || mode > 2 ||
        (mode != 0 && (!log || len < 1)))
        return WM_ERR_INVALID;
    SolveDev &S = b->host[slot];
    S.dt_log = mode ? log : nullptr;
    S.dt_log_len = mode ? len : 0;
    S.dt_mode = mode;
    b->dirty = true;
    return WM_OK;
}

int wm_batch_profile(wm_batch *b, int enable)
{
    if (!b) return WM_ERR_INVALID;
    if (b->prof_on != (enable != 0)) {  // the counters' address is a kernel argument: re-capture
        b->prof_on = enable != 0;
        if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->graph_exec = nullptr;
        b->graph = nullptr;
    }
    return WM_OK;
}

int wm_batch_profile_read(wm_batch *b, double *ms, int reset, void *stream)
{
    if (!b || !ms) return WM_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned long long raw[kPhaseSlots];
    cudaError_t e = cudaMemcpyAsync(raw, b->prof, sizeof raw, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && reset) e = cudaMemsetAsync(b->prof, 0, sizeof raw, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_err("wm_batch_profile_read", e);
        return WM_ERR_CUDA;
    }
    for (int k = 0; k < kPhaseSlots; ++k) ms[k] = 1e-6 * (double)raw[k];
    return WM_OK;
}

int wm_batch_info(wm_batch *b, int *ntiles, int *grid, int *graph)
{
    if (!b) return WM_ERR_INVALID;
    if (b->dirty) {
        int rc = rebuild_tiles(b);
        if (rc) return rc;
    }
    if (ntiles) *ntiles = b->ntiles;
    if (grid) *grid = std::max(1, std::min(b->grid, b->ntiles));
    if (graph) *graph = b->graph_exec != nullptr;
    return WM_OK;
}

}  // extern "C"
