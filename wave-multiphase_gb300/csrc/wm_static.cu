// wm_static.cu -- one RHS stage whose workspace is a statically allocated device array.
//
// Some callers cannot allocate device memory: a host application that hands out every byte of
// device memory from its own pool and does not let libraries call cudaMalloc, or a loop that must
// never wait on the allocator. For them wm_rhs_stage_static runs the same stage as wm_rhs_stage
// (same kernels, same arithmetic) without a handle and without allocating: the face fluxes,
// limiter factors and per-cell sensors live in wm_stage_scratch below, a file-scope device array
// sized for grids of at most WM_STATIC_MAX_CELLS padded cells. Every GPU that loads this library
// keeps that array (about 11.3 MiB) until the process exits.
//
// The array is shared by every call on a device and keeps the previous call's contents. Nothing
// in it needs to start at zero: each entry a stage reads is written earlier in the same stage.
// Two calls that overlap on the GPU (different streams, or different host threads) race on it.
// The stage is the plain binary64 form only (WM_PREC_FP64); a WM_PREC_FP32 parameter set is
// refused with its own message.
#include <cuda.h>  // CUcontext only; the two driver calls are reached through the runtime

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/wavemp.h"
#include "wm_kernels.cuh"

namespace wm {
void set_error_text(const char *msg);  // wm_capi.cu: the text returned by wm_last_error()
}

using namespace wm;

namespace {

constexpr int kArrays = 45;  // 28 face arrays, 3 limiter factors, 11 per-cell arrays, the binary32
                             // entropy of the switch pre-check (in a binary64-sized slot), and two
                             // slots for four binary32 arrays of its pairs
constexpr size_t kArrayBytes = ((size_t)WM_STATIC_MAX_CELLS * sizeof(double) + 255) / 256 * 256;
constexpr size_t kFinBytes = ((size_t)WM_STATIC_MAX_CELLS + 255) / 256 * 256;  // finiteness bytes
constexpr size_t kScratchBytes = (size_t)kArrays * kArrayBytes + 2 * kFinBytes;

static __device__ __align__(256) unsigned char wm_stage_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
struct ScratchSlot {
    unsigned long long ctx_id;  // unique id of the context the address belongs to (0: none yet)
    void *addr;
};
ScratchSlot g_scratch[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// The driver's cuCtxGetCurrent / cuCtxGetId, reached through the runtime (no link to libcuda).
// A context id is unique for the life of the process: after cudaDeviceReset the device's new
// primary context has a new id, its module (and so wm_stage_scratch) may sit at a new address,
// and the address is looked up again.
typedef int (*CtxGetCurrentFn)(CUcontext *);
typedef int (*CtxGetIdFn)(CUcontext, unsigned long long *);

unsigned long long current_context_id()
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult qa = cudaDriverEntryPointSymbolNotFound, qb = qa;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) ==
                cudaSuccess && qa == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) ==
                cudaSuccess && qb == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<CtxGetCurrentFn>(a);
            get_id = reinterpret_cast<CtxGetIdFn>(b);
        }
    });
    if (!get_current || !get_id) return 0;  // unknown: the caller looks the address up each call
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// Device address of wm_stage_scratch on the current device. The host-side name of the array is
// only a stand-in for it, so the address is looked up with that device current: once per device
// and context (again after a cudaDeviceReset), or on every call where the context id is not
// available.
int scratch_address(void **out)
{
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        set_error_text("wm_rhs_stage_static: no usable current CUDA device");
        return WM_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    unsigned long long id = current_context_id();
    if (id == 0 || g_scratch[dev].ctx_id != id || !g_scratch[dev].addr) {
        void *p = nullptr;
        err = cudaGetSymbolAddress(&p, wm_stage_scratch);
        if (err != cudaSuccess || !p) {
            char msg[256];
            snprintf(msg, sizeof msg, "wm_rhs_stage_static: cudaGetSymbolAddress failed: %s",
                     cudaGetErrorString(err));
            set_error_text(msg);
            return WM_ERR_CUDA;
        }
        // the lookup makes the device's primary context current if it was not yet
        g_scratch[dev].ctx_id = id ? id : current_context_id();
        g_scratch[dev].addr = p;
        *out = p;
        return WM_OK;
    }
    *out = g_scratch[dev].addr;
    return WM_OK;
}

bool params_ok(const wm_params *p, int nx, int ny, int g)
{
    if (!p || nx < 1 || ny < 1 || g < 4 || g > 64) return false;
    if (!(p->gamma1 > 1.0) || !(p->gamma2 > 1.0) || !(p->dx > 0.0) || !(p->dy > 0.0)) return false;
    if (!std::isfinite(p->pinf1) || !std::isfinite(p->pinf2) || !(p->cfl > 0.0)) return false;
    if (p->variant != WM_VARIANT_SC && p->variant != WM_VARIANT_M10) return false;
    if (p->recon != WM_RECON_SHIPPED && p->recon != WM_RECON_MP5C6) return false;
    for (int k = 0; k < 4; ++k)
        if (p->bc[k] != WM_BC_TRANSMISSIVE && p->bc[k] != WM_BC_SLIP) return false;
    return true;
}

bool fields_ok(const wm_fields *q, int nyg, bool need_prims)
{
    if (!q || q->pitch < nyg) return false;
    double *const f[10] = {q->ar1, q->ar2, q->ru, q->rv, q->E, q->al, q->u_p, q->v_p, q->p_p, q->al_prim};
    for (int c = 0; c < (need_prims ? 10 : 6); ++c)
        if (!f[c] || ((uintptr_t)f[c] & 7u)) return false;
    return true;
}

Fields fields_of(const wm_fields *q)
{
    Fields F;
    F.f[0] = q->ar1; F.f[1] = q->ar2; F.f[2] = q->ru; F.f[3] = q->rv; F.f[4] = q->E; F.f[5] = q->al;
    F.f[6] = q->u_p; F.f[7] = q->v_p; F.f[8] = q->p_p; F.f[9] = q->al_prim;
    F.pitch = q->pitch;
    return F;
}

}  // namespace

extern "C" int wm_rhs_stage_static(const wm_params *p, int nx, int ny, int g, const wm_fields *q,
                                   const wm_fields *q_old, double dt, double alpha, double beta,
                                   void *stream)
{
    if (p && p->precision == WM_PREC_FP32) {
        // the precision form's workspace (binary32 copies of the state and fluxes) has a different
        // layout; this entry point carries only the plain form's
        set_error_text("wm_rhs_stage_static: the binary64 form only (precision must be WM_PREC_FP64); "
                       "use wm_create + wm_rhs_stage for WM_PREC_FP32");
        return WM_ERR_INVALID;
    }
    if (!params_ok(p, nx, ny, g) || p->precision != WM_PREC_FP64) {
        set_error_text("wm_rhs_stage_static: invalid parameters");
        return WM_ERR_INVALID;
    }
    const long long cells = (long long)(nx + 2 * g) * (long long)(ny + 2 * g);
    if (cells > (long long)WM_STATIC_MAX_CELLS) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "wm_rhs_stage_static: grid of %lld padded cells exceeds the static scratch limit "
                 "of %d padded cells; use wm_create + wm_rhs_stage",
                 cells, (int)WM_STATIC_MAX_CELLS);
        set_error_text(msg);
        return WM_ERR_INVALID;
    }
    if (!fields_ok(q, ny + 2 * g, true) || !std::isfinite(dt) || !std::isfinite(alpha) ||
        !std::isfinite(beta) || (alpha != 0.0 && !fields_ok(q_old, ny + 2 * g, false))) {
        set_error_text("wm_rhs_stage_static: invalid field pointers, pitch or coefficients");
        return WM_ERR_INVALID;
    }
    void *base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;

    Grid G;
    G.nx = nx; G.ny = ny; G.g = g; G.nxg = nx + 2 * g; G.nyg = ny + 2 * g; G.pitch = G.nyg;
    G.dx = p->dx; G.dy = p->dy; G.inv_dx = 1.0 / p->dx; G.inv_dy = 1.0 / p->dy; G.inv_dxf = float(G.inv_dx); G.inv_dyf = float(G.inv_dy); G.cfl = p->cfl;
    const Eos E = make_eos(p->gamma1, p->pinf1, p->gamma2, p->pinf2);

    double *arr[kArrays];
    for (int a = 0; a < kArrays; ++a)
        arr[a] = reinterpret_cast<double *>(static_cast<unsigned char *>(base) + (size_t)a * kArrayBytes);
    Face7 fh, gh, fl, gl;
    for (int c = 0; c < 7; ++c) {
        fh.f[c] = arr[c];
        gh.f[c] = arr[7 + c];
        fl.f[c] = arr[14 + c];
        gl.f[c] = arr[21 + c];
    }
    fl.fin = static_cast<unsigned char *>(base) + (size_t)kArrays * kArrayBytes;
    gl.fin = fl.fin + kFinBytes;
    double *theta[3] = {arr[28], arr[29], arr[30]};
    Prep P;
    P.sx = arr[31]; P.sy = arr[32]; P.ent = arr[33]; P.cx = arr[34]; P.cy = arr[35];
    P.lu = arr[36]; P.lv = arr[37]; P.lp = arr[38]; P.la = arr[39]; P.lc = arr[40]; P.lE = arr[41];
    P.ent64 = arr[33];
    P.ent32 = reinterpret_cast<float *>(arr[42]);
    set_pairs(P.pair, reinterpret_cast<float *>(arr[33]), (size_t)G.nxg * (size_t)G.nyg,
              reinterpret_cast<char *>(arr[43]), kArrayBytes / 2, nullptr);
    Counters none = {nullptr, nullptr, nullptr, nullptr};

    Fields F = fields_of(q), O = alpha != 0.0 ? fields_of(q_old) : F;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    launch_bc(G, p->bc, F, nullptr, s);
    launch_prep(G, E, F, P, p->variant, s);
    launch_faces(G, E, p->variant, p->recon, F, P, fh, gh, fl, gl, true, true, s);
    launch_limiter(G, E, F, Cells32{}, fh, gh, fl, gl, theta, dt, nullptr, none, false, s);
    unsigned flags = FIN_RK3 | FIN_PRIM;
    if (p->emergency_repair) flags |= FIN_ADMISSIBLE;
    if (alpha != 0.0) flags |= FIN_OLD_READ;
    launch_final(G, E, flags, F, O, fh, gh, fl, gl, theta, false, dt, nullptr, alpha, beta, none, s);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof msg, "wm_rhs_stage_static: %s", cudaGetErrorString(err));
        set_error_text(msg);
        return WM_ERR_CUDA;
    }
    return WM_OK;
}
