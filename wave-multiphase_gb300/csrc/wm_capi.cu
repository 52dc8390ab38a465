// wm_capi.cu -- the C ABI of include/wavemp.h: handle, workspace layout and the launch sequences
// of the reference's closures (SC:1894-1995) and of the fused stage / step.
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/wavemp.h"
#include "wm_kernels.cuh"

using namespace wm;

namespace {

thread_local char g_last_error[512] = "";

void set_error(const char *where, cudaError_t err)
{
    snprintf(g_last_error, sizeof g_last_error, "%s: %s", where, cudaGetErrorString(err));
}

int check_launch(const char *where)
{
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        set_error(where, err);
        return WM_ERR_CUDA;
    }
    return WM_OK;
}

constexpr int kFaceArrays = 28, kThetaArrays = 3, kPrepArrays = 11;
constexpr int kArrays = kFaceArrays + kThetaArrays + kPrepArrays;
constexpr int kCellCopies = 9;  // binary32 cell copies of the precision form
// The switch pre-check's binary32 pairs (PrepT::pair) beyond the density pair, which overlays the
// binary64 entropy: pressure hi and lo and gamma hi and lo; the precision form's pressure hi is its
// binary32 pressure copy.
constexpr int kPairArrays64 = 4, kPairArrays32 = 3;
constexpr size_t kAlign = 256;
constexpr size_t kTailBytes = 256;  // counters and dt slots

size_t array_bytes(int nx, int ny, int g, size_t elem = sizeof(double))
{
    size_t n = (size_t)(nx + 2 * g) * (size_t)(ny + 2 * g) * elem;
    return (n + kAlign - 1) / kAlign * kAlign;
}

// Workspace of the plain form: 42 binary64 arrays, the binary32 entropy of the switch pre-check and
// 4 binary32 arrays of its pairs. Precision form: 28 binary32 face arrays, 3
// binary32 limiter factors (bound solves in binary64, stored in the flux type), 11 binary32
// per-cell arrays, 9 binary32 cell copies, the binary64 entropy of the binary64 switches and 3
// binary32 arrays of the pairs.
// Both: then the first-order sweeps' per-face finiteness bytes (x, y), one byte a padded cell each.
size_t layout_bytes(int precision, int nx, int ny, int g)
{
    const size_t fin = 2 * array_bytes(nx, ny, g, 1);
    if (precision == WM_PREC_FP32)
        return (size_t)(kArrays + kCellCopies + kPairArrays32) * array_bytes(nx, ny, g, sizeof(float)) +
               array_bytes(nx, ny, g) + fin + kTailBytes;
    return (size_t)kArrays * array_bytes(nx, ny, g) + (size_t)(1 + kPairArrays64) * array_bytes(nx, ny, g, sizeof(float)) +
           fin + kTailBytes;
}

bool valid_params(const wm_params *p, int nx, int ny, int g)
{
    if (!p || nx < 1 || ny < 1 || g < 4 || g > 64) return false;
    if (!(p->gamma1 > 1.0) || !(p->gamma2 > 1.0) || !(p->dx > 0.0) || !(p->dy > 0.0)) return false;
    if (!std::isfinite(p->pinf1) || !std::isfinite(p->pinf2) || !(p->cfl > 0.0)) return false;
    if (p->variant != WM_VARIANT_SC && p->variant != WM_VARIANT_M10) return false;
    if (p->recon != WM_RECON_SHIPPED && p->recon != WM_RECON_MP5C6) return false;
    if (p->precision != WM_PREC_FP64 && p->precision != WM_PREC_FP32) return false;
    for (int k = 0; k < 4; ++k)
        if (p->bc[k] != WM_BC_TRANSMISSIVE && p->bc[k] != WM_BC_SLIP) return false;
    if ((double)(nx + 2 * g) * (double)(ny + 2 * g) > 4.0e9) return false;
    return true;
}

}  // namespace

namespace wm {
// Sets the text returned by wm_last_error() (used by entry points defined in other files).
void set_error_text(const char *msg) { snprintf(g_last_error, sizeof g_last_error, "%s", msg); }
}  // namespace wm

// Device-resident state of wm_run's loop: the caller's schedule plus the loop's own counters.
struct RunClock {
    wm_schedule s;
    long long iter, max_iter;
    double dt_use;  // the dt of the step in flight (after the save-time and end-time clamps)
};

struct wm_handle {
    wm_params P;
    Grid g;
    Eos e;
    void *ws = nullptr;
    bool own_ws = false;
    bool fp32 = false;
    double *arr[kArrays];  // binary64 arrays (plain form) by WM_WS_* index
    float *arr32[kArrays]; // binary32 arrays (precision form) by WM_WS_* index
    Face7 fh, gh, fl, gl;
    Face<float> fh32, gh32, fl32, gl32;
    double *theta[3];
    float *theta32[3];
    Prep prep;
    PrepT<float> prep32;
    Cells32 cells32;
    Counters cnt;
    unsigned long long *ctr_base = nullptr;
    double *dt_dev[2];
    int dt_cur = 0;
    bool dt_valid = false;
    long long steps = 0;
    bool fluxes_ready = false, low_ready = false;
    bool defer_limiter = false;  // fused stage: limiter blends rebuilt in registers (wm_set_limiter_sweeps)
    bool prechecks = true;       // precision form: binary32 pre-checks of binary64 tests (wm_set_prechecks)
    bool sw64 = false;           // precision form: binary64 switches (wm_params.fp64_switches)
    // device-side time loop (wm_run): clock block, graph with a conditional while node
    struct RunClock *clock = nullptr;
    cudaGraph_t run_graph = nullptr;
    cudaGraphExec_t run_exec = nullptr;
    bool run_graph_ok = true;
    Fields run_F{}, run_O{};
    // kernel-group profiler (wm_profile)
    bool prof = false;
    struct Rec {
        int group, launches;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    double prof_ms[WM_PROF_GROUPS] = {0};
    long long prof_n[WM_PROF_GROUPS] = {0};
};

namespace {

cudaEvent_t take_event(wm_handle *h)
{
    if (!h->pool.empty()) {
        cudaEvent_t e = h->pool.back();
        h->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Brackets a group of launches with events when the profiler is on.
struct ProfScope {
    wm_handle *h;
    int group, launches;
    cudaStream_t s;
    cudaEvent_t a = nullptr;
    ProfScope(wm_handle *h_, int g, int n, cudaStream_t s_) : h(h_), group(g), launches(n), s(s_)
    {
        if (h->prof) {
            a = take_event(h);
            cudaEventRecord(a, s);
        }
    }
    ~ProfScope()
    {
        if (h->prof && a) {
            cudaEvent_t b = take_event(h);
            cudaEventRecord(b, s);
            h->recs.push_back({group, launches, a, b});
        }
    }
};

}  // namespace

namespace {

bool fields_ok(const wm_handle *h, const wm_fields *q, bool need_prims = true)
{
    if (!q || q->pitch < h->g.nyg) return false;
    double *const f[10] = {q->ar1, q->ar2, q->ru, q->rv, q->E, q->al, q->u_p, q->v_p, q->p_p, q->al_prim};
    for (int c = 0; c < (need_prims ? 10 : 6); ++c)
        if (!f[c] || ((uintptr_t)f[c] & 7u)) return false;
    return true;
}

Fields to_fields(const wm_fields *q)
{
    Fields F;
    F.f[0] = q->ar1; F.f[1] = q->ar2; F.f[2] = q->ru; F.f[3] = q->rv; F.f[4] = q->E; F.f[5] = q->al;
    F.f[6] = q->u_p; F.f[7] = q->v_p; F.f[8] = q->p_p; F.f[9] = q->al_prim;
    F.pitch = q->pitch;
    return F;
}

cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

unsigned final_flags(const wm_handle *h, double alpha)
{
    unsigned fl = FIN_RK3 | FIN_PRIM;
    if (h->P.emergency_repair) fl |= FIN_ADMISSIBLE;
    if (alpha != 0.0) fl |= FIN_OLD_READ;
    return fl;
}

}  // namespace

extern "C" {

const char *wm_version(void) { return "wavemp 0.2 (sm_103a; fp64 plain and fp32 precision forms)"; }
const char *wm_last_error(void) { return g_last_error; }

size_t wm_workspace_bytes(const wm_params *p, int nx, int ny, int g)
{
    if (!valid_params(p, nx, ny, g)) return 0;
    return layout_bytes(p->precision, nx, ny, g);
}

int wm_create(const wm_params *p, int nx, int ny, int g, void *workspace, size_t workspace_bytes,
              wm_handle **out)
{
    if (!out) return WM_ERR_INVALID;
    *out = nullptr;
    if (!valid_params(p, nx, ny, g)) return WM_ERR_INVALID;
    size_t need = wm_workspace_bytes(p, nx, ny, g);
    if (workspace && (workspace_bytes < need || ((uintptr_t)workspace % kAlign))) return WM_ERR_NOMEM;
    wm_handle *h = new (std::nothrow) wm_handle();
    if (!h) return WM_ERR_NOMEM;
    h->P = *p;
    Grid &G = h->g;
    G.nx = nx; G.ny = ny; G.g = g; G.nxg = nx + 2 * g; G.nyg = ny + 2 * g; G.pitch = G.nyg;
    G.dx = p->dx; G.dy = p->dy; G.inv_dx = 1.0 / p->dx; G.inv_dy = 1.0 / p->dy; G.inv_dxf = float(G.inv_dx); G.inv_dyf = float(G.inv_dy); G.cfl = p->cfl;
    h->e = make_eos(p->gamma1, p->pinf1, p->gamma2, p->pinf2);

    if (workspace) {
        h->ws = workspace;
    } else {
        cudaError_t err = cudaMalloc(&h->ws, need);
        if (err != cudaSuccess) {
            set_error("wm_create cudaMalloc", err);
            delete h;
            return WM_ERR_NOMEM;
        }
        h->own_ws = true;
    }
    cudaError_t err = cudaMemset(h->ws, 0, need);
    if (err != cudaSuccess) {
        set_error("wm_create cudaMemset", err);
        if (h->own_ws) cudaFree(h->ws);
        delete h;
        return WM_ERR_CUDA;
    }
    char *base = static_cast<char *>(h->ws);
    const size_t cells = (size_t)(nx + 2 * g) * (size_t)(ny + 2 * g);
    char *tail;
    h->fp32 = p->precision == WM_PREC_FP32;
    // measured on the triple point: rebuilding the blends in registers pays in binary32 (1525 ->
    // 1818 Mcell-stage/s) and costs in binary64 (254 -> 229), whose pipe is the bound there
    h->defer_limiter = h->fp32;
    if (!h->fp32) {
        size_t ab = array_bytes(nx, ny, g);
        for (int a = 0; a < kArrays; ++a) h->arr[a] = reinterpret_cast<double *>(base + (size_t)a * ab);
        for (int c = 0; c < 7; ++c) {
            h->fh.f[c] = h->arr[WM_WS_FX + c];
            h->gh.f[c] = h->arr[WM_WS_GY + c];
            h->fl.f[c] = h->arr[WM_WS_FXL + c];
            h->gl.f[c] = h->arr[WM_WS_GYL + c];
        }
        for (int s = 0; s < 3; ++s) h->theta[s] = h->arr[WM_WS_THETA + s];
        Prep &P = h->prep;
        P.sx = h->arr[WM_WS_SIGMA_X];
        P.sy = h->arr[WM_WS_SIGMA_Y];
        P.ent = h->arr[33]; P.cx = h->arr[34]; P.cy = h->arr[35];
        P.lu = h->arr[36]; P.lv = h->arr[37]; P.lp = h->arr[38]; P.la = h->arr[39]; P.lc = h->arr[40];
        P.lE = h->arr[41];
        P.ent64 = h->arr[33];
        const size_t ab4 = array_bytes(nx, ny, g, sizeof(float));
        P.ent32 = reinterpret_cast<float *>(base + (size_t)kArrays * ab);
        set_pairs(P.pair, reinterpret_cast<float *>(h->arr[33]), cells, base + (size_t)kArrays * ab + ab4, ab4,
                  nullptr);
        tail = base + (size_t)kArrays * ab + (size_t)(1 + kPairArrays64) * ab4;
        h->fl.fin = reinterpret_cast<unsigned char *>(tail);
        h->gl.fin = h->fl.fin + array_bytes(nx, ny, g, 1);
        tail += 2 * array_bytes(nx, ny, g, 1);
    } else {
        size_t ab4 = array_bytes(nx, ny, g, sizeof(float));
        char *cur = base;
        for (int a = 0; a < kArrays; ++a) {
            h->arr32[a] = reinterpret_cast<float *>(cur);
            h->arr[a] = nullptr;
            cur += ab4;
        }
        float *copies[kCellCopies];
        for (int c = 0; c < kCellCopies; ++c) {
            copies[c] = reinterpret_cast<float *>(cur);
            cur += ab4;
        }
        double *ent64 = reinterpret_cast<double *>(cur);
        cur += array_bytes(nx, ny, g);
        char *pairs = cur;
        cur += (size_t)kPairArrays32 * ab4;
        h->sw64 = p->fp64_switches != 0;
        for (int c = 0; c < 7; ++c) {
            h->fh32.f[c] = h->arr32[WM_WS_FX + c];
            h->gh32.f[c] = h->arr32[WM_WS_GY + c];
            h->fl32.f[c] = h->arr32[WM_WS_FXL + c];
            h->gl32.f[c] = h->arr32[WM_WS_GYL + c];
        }
        for (int s = 0; s < 3; ++s) {
            h->theta[s] = nullptr;
            h->theta32[s] = h->arr32[WM_WS_THETA + s];
        }
        PrepT<float> &P = h->prep32;
        P.sx = h->arr32[WM_WS_SIGMA_X];
        P.sy = h->arr32[WM_WS_SIGMA_Y];
        P.ent = h->arr32[33]; P.cx = h->arr32[34]; P.cy = h->arr32[35];
        P.lu = h->arr32[36]; P.lv = h->arr32[37]; P.lp = h->arr32[38]; P.la = h->arr32[39];
        P.lc = h->arr32[40]; P.lE = h->arr32[41];
        P.ent64 = ent64;
        P.ent32 = P.ent;
        Cells32 &C = h->cells32;
        C.ar1 = copies[0]; C.ar2 = copies[1]; C.ru = copies[2]; C.rv = copies[3];
        C.p = copies[4]; C.al = copies[5]; C.u = copies[6]; C.v = copies[7]; C.E = copies[8];
        set_pairs(P.pair, reinterpret_cast<float *>(ent64), cells, pairs, ab4, C.p);
        h->fl32.fin = reinterpret_cast<unsigned char *>(cur);
        h->gl32.fin = h->fl32.fin + array_bytes(nx, ny, g, 1);
        tail = cur + 2 * array_bytes(nx, ny, g, 1);
    }
    h->ctr_base = reinterpret_cast<unsigned long long *>(tail);
    h->cnt.repaired = h->ctr_base + 0;
    h->cnt.nonfinite = h->ctr_base + 1;
    h->cnt.limited = h->ctr_base + 2;
    h->cnt.dt_bits = h->ctr_base + 3;
    h->dt_dev[0] = reinterpret_cast<double *>(tail + 64);
    h->dt_dev[1] = reinterpret_cast<double *>(tail + 72);
    *out = h;
    return WM_OK;
}

void wm_destroy(wm_handle *h)
{
    if (!h) return;
    for (auto &r : h->recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : h->pool) cudaEventDestroy(e);
    if (h->run_exec) cudaGraphExecDestroy(h->run_exec);
    if (h->run_graph) cudaGraphDestroy(h->run_graph);
    if (h->clock) cudaFree(h->clock);
    if (h->own_ws && h->ws) cudaFree(h->ws);
    delete h;
}

int wm_profile(wm_handle *h, int enable)
{
    if (!h) return WM_ERR_INVALID;
    h->prof = enable != 0;
    return WM_OK;
}

int wm_profile_read(wm_handle *h, double ms[WM_PROF_GROUPS], long long launches[WM_PROF_GROUPS],
                    int reset)
{
    if (!h || !ms || !launches) return WM_ERR_INVALID;
    for (auto &r : h->recs) {
        cudaError_t err = cudaEventSynchronize(r.b);
        float t = 0.f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&t, r.a, r.b);
        if (err != cudaSuccess) {
            set_error("wm_profile_read", err);
            return WM_ERR_CUDA;
        }
        h->prof_ms[r.group] += t;
        h->prof_n[r.group] += r.launches;
        h->pool.push_back(r.a);
        h->pool.push_back(r.b);
    }
    h->recs.clear();
    for (int g = 0; g < WM_PROF_GROUPS; ++g) {
        ms[g] = h->prof_ms[g];
        launches[g] = h->prof_n[g];
        if (reset) {
            h->prof_ms[g] = 0.0;
            h->prof_n[g] = 0;
        }
    }
    return WM_OK;
}

int wm_apply_bc(wm_handle *h, const wm_fields *q, void *stream)
{
    if (!h || !fields_ok(h, q)) return WM_ERR_INVALID;
    Fields F = to_fields(q);
    launch_bc(h->g, h->P.bc, F, nullptr, as_stream(stream));
    return check_launch("wm_apply_bc");
}

int wm_compute_fluxes(wm_handle *h, const wm_fields *q, void *stream)
{
    if (!h || !fields_ok(h, q)) return WM_ERR_INVALID;
    Fields F = to_fields(q);
    cudaStream_t s = as_stream(stream);
    if (h->fp32) {
        launch_prep32(h->g, h->e, F, h->prep32, h->cells32, h->P.variant, h->sw64, s, h->prechecks);
        launch_faces32(h->g, h->e, h->P.variant, h->P.recon, h->cells32, h->prep32, h->fh32, h->gh32,
                       h->fl32, h->gl32, true, false, s);
    } else {
        launch_prep(h->g, h->e, F, h->prep, h->P.variant, s, h->prechecks);
        launch_faces(h->g, h->e, h->P.variant, h->P.recon, F, h->prep, h->fh, h->gh, h->fl, h->gl,
                     true, false, s);
    }
    h->fluxes_ready = true;
    return check_launch("wm_compute_fluxes");
}

int wm_compute_low_fluxes(wm_handle *h, const wm_fields *q, void *stream)
{
    if (!h || !fields_ok(h, q)) return WM_ERR_INVALID;
    Fields F = to_fields(q);
    cudaStream_t s = as_stream(stream);
    if (h->fp32) {
        launch_prep32(h->g, h->e, F, h->prep32, h->cells32, h->P.variant, h->sw64, s, h->prechecks);
        launch_faces32(h->g, h->e, h->P.variant, h->P.recon, h->cells32, h->prep32, h->fh32, h->gh32,
                       h->fl32, h->gl32, false, true, s);
    } else {
        launch_prep(h->g, h->e, F, h->prep, h->P.variant, s, h->prechecks);
        launch_faces(h->g, h->e, h->P.variant, h->P.recon, F, h->prep, h->fh, h->gh, h->fl, h->gl,
                     false, true, s);
    }
    h->low_ready = true;
    return check_launch("wm_compute_low_fluxes");
}

int wm_limit_fluxes(wm_handle *h, const wm_fields *q, double dt, void *stream)
{
    if (!h || !fields_ok(h, q) || !std::isfinite(dt)) return WM_ERR_INVALID;
    if (!h->fluxes_ready || !h->low_ready) return WM_ERR_STATE;
    if (h->fp32)
        launch_limiter(h->g, h->e, to_fields(q), h->cells32, h->fh32, h->gh32, h->fl32, h->gl32, h->theta32, dt,
                       nullptr, h->cnt, false, as_stream(stream), nullptr, h->prechecks);
    else
        launch_limiter(h->g, h->e, to_fields(q), Cells32{}, h->fh, h->gh, h->fl, h->gl, h->theta, dt, nullptr,
                       h->cnt, false, as_stream(stream), nullptr, h->prechecks);
    return check_launch("wm_limit_fluxes");
}

int wm_rk3_update(wm_handle *h, const wm_fields *q, const wm_fields *q_old, double alpha,
                  double beta, double dt, void *stream)
{
    if (!h || !fields_ok(h, q) || !std::isfinite(dt)) return WM_ERR_INVALID;
    if (alpha != 0.0 && !fields_ok(h, q_old, false)) return WM_ERR_INVALID;
    if (!h->fluxes_ready) return WM_ERR_STATE;
    Fields F = to_fields(q), O = q_old ? to_fields(q_old) : F;
    const unsigned fl = FIN_RK3 | (alpha != 0.0 ? FIN_OLD_READ : 0u);
    if (h->fp32)
        launch_final(h->g, h->e, fl, F, O, h->fh32, h->gh32, h->fl32, h->gl32, h->theta32, false, dt,
                     nullptr, alpha, beta, h->cnt, as_stream(stream));
    else
        launch_final(h->g, h->e, fl, F, O, h->fh, h->gh, h->fl, h->gl, h->theta, false, dt, nullptr,
                     alpha, beta, h->cnt, as_stream(stream));
    return check_launch("wm_rk3_update");
}

int wm_enforce_admissible(wm_handle *h, const wm_fields *q, void *stream)
{
    if (!h || !fields_ok(h, q)) return WM_ERR_INVALID;
    if (!h->P.emergency_repair) return WM_OK;
    Fields F = to_fields(q);
    launch_final(h->g, h->e, FIN_ADMISSIBLE, F, F, h->fh, h->gh, h->fl, h->gl, h->theta, false, 0.0,
                 nullptr, 0.0, 1.0, h->cnt, as_stream(stream));
    return check_launch("wm_enforce_admissible");
}

int wm_update_prims(wm_handle *h, const wm_fields *q, void *stream)
{
    if (!h || !fields_ok(h, q)) return WM_ERR_INVALID;
    Fields F = to_fields(q);
    launch_final(h->g, h->e, FIN_PRIM, F, F, h->fh, h->gh, h->fl, h->gl, h->theta, false, 0.0, nullptr,
                 0.0, 1.0, h->cnt, as_stream(stream));
    return check_launch("wm_update_prims");
}

int wm_copy_old(wm_handle *h, const wm_fields *q, const wm_fields *q_old, void *stream)
{
    if (!h || !fields_ok(h, q, false) || !fields_ok(h, q_old, false)) return WM_ERR_INVALID;
    launch_copy_old(h->g, to_fields(q), to_fields(q_old), as_stream(stream));
    return check_launch("wm_copy_old");
}

int wm_init_dt(wm_handle *h, const wm_fields *q, void *stream)
{
    if (!h || !fields_ok(h, q)) return WM_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    launch_dt_reset(h->cnt, s);
    launch_dt_cell(h->g, h->e, to_fields(q), h->cnt, s);
    launch_dt_finalize(h->g, h->cnt, h->dt_dev[h->dt_cur], s);
    h->dt_valid = true;
    return check_launch("wm_init_dt");
}

int wm_get_dt(wm_handle *h, const wm_fields *q, double *dt, void *stream)
{
    if (!dt) return WM_ERR_INVALID;
    int rc = wm_init_dt(h, q, stream);
    if (rc) return rc;
    cudaStream_t s = as_stream(stream);
    cudaError_t err = cudaMemcpyAsync(dt, h->dt_dev[h->dt_cur], sizeof(double), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) {
        set_error("wm_get_dt", err);
        return WM_ERR_CUDA;
    }
    return WM_OK;
}

// The binary64 form's first-order faces for the fused stage: the sweep writes only their finiteness
// bytes, and the limiter's bound solve and blends form the values they read from the stage state's
// partial densities and the preparation pass's first-order cell states (Face::src).
static void on_demand_low(const wm_handle *h, const Fields &F, Face<double> &fl, Face<double> &gl)
{
    fl = h->fl;
    gl = h->gl;
    LowSrc s;
    s.ar1 = F.f[F_AR1];
    s.ar2 = F.f[F_AR2];
    s.pitch = F.pitch;
    s.lu = h->prep.lu; s.lv = h->prep.lv; s.lp = h->prep.lp;
    s.la = h->prep.la; s.lc = h->prep.lc; s.lE = h->prep.lE;
    s.nyg = h->g.nyg;
    s.on = 1;
    fl.src = s;
    gl.src = s;
}

// One stage; `save_old` fuses copy_old, `dt_dev` (when non-null) replaces dt, `want_dt` appends
// the time-step reduction of the updated state.
static int run_stage(wm_handle *h, const Fields &F, const Fields &O, double dt, const double *dt_dev,
                     double alpha, double beta, bool save_old, bool want_dt, cudaStream_t s)
{
    {
        ProfScope ps(h, WM_PROF_BC, 2, s);
        launch_bc(h->g, h->P.bc, F, save_old ? &O : nullptr, s);
    }
    {
        ProfScope ps(h, WM_PROF_PREP, 2, s);
        if (h->fp32)
            launch_prep32(h->g, h->e, F, h->prep32, h->cells32, h->P.variant, h->sw64, s, h->prechecks);
        else
            launch_prep(h->g, h->e, F, h->prep, h->P.variant, s, h->prechecks);
    }
    // binary64 with blends in place: first-order values formed on demand; with deferred blends the
    // passes and the combine rebuild the blends from the stored values
    const bool on_demand = !h->fp32 && !h->defer_limiter;
    Face<double> fl = h->fl, gl = h->gl;
    if (on_demand) on_demand_low(h, F, fl, gl);
    {
        ProfScope ps(h, WM_PROF_FACES, 2, s);
        if (h->fp32)
            launch_faces32(h->g, h->e, h->P.variant, h->P.recon, h->cells32, h->prep32, h->fh32,
                           h->gh32, h->fl32, h->gl32, true, true, s);
        else
            launch_faces(h->g, h->e, h->P.variant, h->P.recon, F, h->prep, h->fh, h->gh, fl, gl, true, true, s);
    }
    {
        ProfScope ps(h, WM_PROF_LIMITER, h->defer_limiter ? 3 : 6, s);
        if (h->fp32)
            launch_limiter(h->g, h->e, F, h->cells32, h->fh32, h->gh32, h->fl32, h->gl32, h->theta32, dt, dt_dev,
                           h->cnt, h->defer_limiter, s, nullptr, h->prechecks);
        else
            launch_limiter(h->g, h->e, F, Cells32{}, h->fh, h->gh, fl, gl, h->theta, dt, dt_dev, h->cnt,
                           h->defer_limiter, s, nullptr, h->prechecks);
    }
    unsigned flags = final_flags(h, alpha);
    if (!h->prechecks) flags |= FIN_EXACT_CHECKS;
    if (save_old) flags |= FIN_SAVE_OLD;
    {
        ProfScope ps(h, WM_PROF_FINAL, want_dt ? 2 : 1, s);
        if (want_dt) {
            flags |= FIN_DT;
            launch_dt_reset(h->cnt, s);
        }
        if (h->fp32)
            launch_final(h->g, h->e, flags, F, O, h->fh32, h->gh32, h->fl32, h->gl32, h->theta32,
                         h->defer_limiter, dt, dt_dev, alpha, beta, h->cnt, s);
        else
            launch_final(h->g, h->e, flags, F, O, h->fh, h->gh, h->fl, h->gl, h->theta, h->defer_limiter,
                         dt, dt_dev, alpha, beta, h->cnt, s);
    }
    h->fluxes_ready = true;
    h->low_ready = !on_demand;  // formed on demand: the first-order arrays are left unwritten
    return check_launch("stage");
}

int wm_rhs_stage(wm_handle *h, const wm_fields *q, const wm_fields *q_old, double dt, double alpha,
                 double beta, void *stream)
{
    if (!h || !fields_ok(h, q) || !std::isfinite(dt) || !std::isfinite(alpha) || !std::isfinite(beta))
        return WM_ERR_INVALID;
    if (alpha != 0.0 && !fields_ok(h, q_old, false)) return WM_ERR_INVALID;
    Fields F = to_fields(q), O = (alpha != 0.0) ? to_fields(q_old) : F;
    return run_stage(h, F, O, dt, nullptr, alpha, beta, false, false, as_stream(stream));
}

int wm_step(wm_handle *h, const wm_fields *q, const wm_fields *q_old, double dt, double *dt_next,
            void *stream)
{
    if (!h || !fields_ok(h, q) || !fields_ok(h, q_old, false) || std::isnan(dt)) return WM_ERR_INVALID;
    if (!(dt > 0.0) && !h->dt_valid) return WM_ERR_STATE;
    cudaStream_t s = as_stream(stream);
    Fields F = to_fields(q), O = to_fields(q_old);
    const double *dd = dt > 0.0 ? nullptr : h->dt_dev[h->dt_cur];
    int rc = run_stage(h, F, O, dt, dd, 0.0, 1.0, true, false, s);
    if (!rc) rc = run_stage(h, F, O, dt, dd, 0.75, 0.25, false, false, s);
    if (!rc) rc = run_stage(h, F, O, dt, dd, 1.0 / 3.0, 2.0 / 3.0, false, true, s);
    if (rc) return rc;
    int nxt = 1 - h->dt_cur;
    {
        ProfScope ps(h, WM_PROF_FINAL, 1, s);
        launch_dt_finalize(h->g, h->cnt, h->dt_dev[nxt], s);
    }
    h->dt_cur = nxt;
    h->dt_valid = true;
    h->steps++;
    rc = check_launch("wm_step");
    if (rc) return rc;
    if (dt_next) {
        cudaError_t err = cudaMemcpyAsync(dt_next, h->dt_dev[h->dt_cur], sizeof(double),
                                          cudaMemcpyDeviceToHost, s);
        if (err == cudaSuccess) err = cudaStreamSynchronize(s);
        if (err != cudaSuccess) {
            set_error("wm_step dt", err);
            return WM_ERR_CUDA;
        }
    }
    return WM_OK;
}

}  // extern "C"

namespace {

// The dt clamps at the top of the reference's loop (SC:2021-2026): to each save time not yet
// written, then to the end time.
__global__ void run_clamp_kernel(RunClock *c, const double *dt_cfl)
{
    double dt = *dt_cfl;
    const double t = c->s.t;
    for (int k = 0; k < c->s.nsaves; ++k)
        if (!c->s.saved[k] && t + dt > c->s.save_times[k]) dt = c->s.save_times[k] - t;
    if (t + dt > c->s.t_end) dt = c->s.t_end - t;
    c->dt_use = dt;
}

// The bottom of the loop (SC:2057-2073): time and step advance, the next dt is the CFL dt just
// reduced, a save time is reached when |t - ts| < dt/2 with that dt, the loop runs while
// t < t_end - 1e-14. The graph's while node repeats the step until a save time is reached, the end
// time, or the call's step limit.
__global__ void run_advance_kernel(RunClock *c, const double *dt_cfl, cudaGraphConditionalHandle cond,
                                   int in_graph)
{
    const double t = c->s.t + c->dt_use;
    c->s.t = t;
    c->s.step += 1;
    c->iter += 1;
    const double dt = *dt_cfl;
    c->s.dt = dt;
    int hit = -1;
    for (int k = 0; k < c->s.nsaves; ++k) {
        if (!c->s.saved[k] && fabs(t - c->s.save_times[k]) < 0.5 * dt) {
            c->s.saved[k] = 1;
            if (hit < 0) hit = k;
        }
    }
    c->s.hit = hit;
    c->s.finished = !(t < c->s.t_end - 1.0e-14);
    const bool go = hit < 0 && !c->s.finished && c->iter < c->max_iter;
    if (in_graph) cudaGraphSetConditional(cond, go ? 1u : 0u);
}

double *clock_dt_use(wm_handle *h)
{
    return reinterpret_cast<double *>(reinterpret_cast<char *>(h->clock) + offsetof(RunClock, dt_use));
}

// One loop iteration: clamp, three stages on the clamped dt, CFL reduction into dt slot 0, advance.
int run_iteration(wm_handle *h, const Fields &F, const Fields &O, cudaGraphConditionalHandle cond,
                  int in_graph, cudaStream_t s)
{
    run_clamp_kernel<<<1, 1, 0, s>>>(h->clock, h->dt_dev[0]);
    const double *dd = clock_dt_use(h);
    int rc = run_stage(h, F, O, 0.0, dd, 0.0, 1.0, true, false, s);
    if (!rc) rc = run_stage(h, F, O, 0.0, dd, 0.75, 0.25, false, false, s);
    if (!rc) rc = run_stage(h, F, O, 0.0, dd, 1.0 / 3.0, 2.0 / 3.0, false, true, s);
    if (rc) return rc;
    launch_dt_finalize(h->g, h->cnt, h->dt_dev[0], s);
    run_advance_kernel<<<1, 1, 0, s>>>(h->clock, h->dt_dev[0], cond, in_graph);
    return check_launch("wm_run step");
}

void drop_run_graph(wm_handle *h)
{
    if (h->run_exec) cudaGraphExecDestroy(h->run_exec);
    if (h->run_graph) cudaGraphDestroy(h->run_graph);
    h->run_exec = nullptr;
    h->run_graph = nullptr;
}

// Graph: one conditional while node whose body is one loop iteration (captured into the body).
bool build_run_graph(wm_handle *h, const Fields &F, const Fields &O)
{
    drop_run_graph(h);
    cudaGraph_t g = nullptr;
    cudaStream_t cs = nullptr;
    bool ok = cudaGraphCreate(&g, 0) == cudaSuccess;
    cudaGraphConditionalHandle cond = 0;
    if (ok) ok = cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (ok) ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) == cudaSuccess;
    if (ok) ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess;
    if (ok) {
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        ok = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
             cudaSuccess;
        if (ok) {
            const bool prof = h->prof;
            h->prof = false;  // no event records inside the body
            int rc = run_iteration(h, F, O, cond, 1, cs);
            h->prof = prof;
            cudaGraph_t out = nullptr;
            ok = cudaStreamEndCapture(cs, &out) == cudaSuccess && rc == WM_OK;
        }
    }
    if (ok) ok = cudaGraphInstantiate(&h->run_exec, g, 0) == cudaSuccess;
    if (cs) cudaStreamDestroy(cs);
    if (ok) {
        h->run_graph = g;
        h->run_F = F;
        h->run_O = O;
    } else {
        if (h->run_exec) cudaGraphExecDestroy(h->run_exec);
        h->run_exec = nullptr;
        if (g) cudaGraphDestroy(g);
    }
    cudaGetLastError();
    return ok;
}

bool same_fields(const Fields &a, const Fields &b) { return memcmp(&a, &b, sizeof(Fields)) == 0; }

}  // namespace

extern "C" {

int wm_run(wm_handle *h, const wm_fields *q, const wm_fields *q_old, wm_schedule *sched, long long max_steps,
           void *stream)
{
    if (!h || !fields_ok(h, q) || !fields_ok(h, q_old, false) || !sched || max_steps < 1 ||
        sched->nsaves < 0 || sched->nsaves > WM_MAX_SAVES || std::isnan(sched->t) || std::isnan(sched->t_end))
        return WM_ERR_INVALID;
    sched->hit = -1;
    if (!(sched->t < sched->t_end - 1.0e-14)) {
        sched->finished = 1;
        return WM_OK;
    }
    cudaStream_t s = as_stream(stream);
    Fields F = to_fields(q), O = to_fields(q_old);
    cudaError_t err = cudaSuccess;
    if (!h->clock) {
        err = cudaMalloc(&h->clock, sizeof(RunClock));
        if (err != cudaSuccess) {
            h->clock = nullptr;
            set_error("wm_run", err);
            return WM_ERR_NOMEM;
        }
    }
    // the loop's dt lives in slot 0: get_dt before the loop (SC:2015), or the dt of the last step
    if (!h->dt_valid) {
        h->dt_cur = 0;
        launch_dt_reset(h->cnt, s);
        launch_dt_cell(h->g, h->e, F, h->cnt, s);
        launch_dt_finalize(h->g, h->cnt, h->dt_dev[0], s);
        h->dt_valid = true;
    } else if (h->dt_cur != 0) {
        err = cudaMemcpyAsync(h->dt_dev[0], h->dt_dev[1], sizeof(double), cudaMemcpyDeviceToDevice, s);
        h->dt_cur = 0;
    }
    RunClock c;
    c.s = *sched;
    c.s.hit = -1;
    c.s.finished = 0;
    c.iter = 0;
    c.max_iter = max_steps;
    c.dt_use = 0.0;
    if (err == cudaSuccess) err = cudaMemcpyAsync(h->clock, &c, sizeof c, cudaMemcpyHostToDevice, s);
    if (err != cudaSuccess) {
        set_error("wm_run", err);
        return WM_ERR_CUDA;
    }
    if (h->run_graph_ok && (!h->run_exec || !same_fields(F, h->run_F) || !same_fields(O, h->run_O)))
        h->run_graph_ok = build_run_graph(h, F, O);
    if (h->run_exec) {
        err = cudaGraphLaunch(h->run_exec, s);
        if (err == cudaSuccess) err = cudaMemcpyAsync(&c, h->clock, sizeof c, cudaMemcpyDeviceToHost, s);
        if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    } else {  // no conditional graphs: the same kernels, one host wait per step
        for (long long n = 0; n < max_steps && err == cudaSuccess; ++n) {
            int rc = run_iteration(h, F, O, 0, 0, s);
            if (rc) return rc;
            err = cudaMemcpyAsync(&c, h->clock, sizeof c, cudaMemcpyDeviceToHost, s);
            if (err == cudaSuccess) err = cudaStreamSynchronize(s);
            if (c.s.hit >= 0 || c.s.finished) break;
        }
    }
    if (err != cudaSuccess) {
        set_error("wm_run", err);
        return WM_ERR_CUDA;
    }
    *sched = c.s;
    h->steps += c.iter;
    return WM_OK;
}

int wm_run_uses_graph(wm_handle *h) { return h && h->run_exec ? 1 : 0; }

int wm_verify_limiter_precheck(wm_handle *h, const wm_fields *q, double dt, long long *decided,
                               long long *disagreed, void *stream)
{
    if (!h || !fields_ok(h, q) || !std::isfinite(dt) || !decided || !disagreed) return WM_ERR_INVALID;
    if (!h->fluxes_ready || !h->low_ready) return WM_ERR_STATE;
    unsigned long long *ctr = nullptr, host[2] = {0, 0};
    cudaStream_t s = as_stream(stream);
    cudaError_t err = cudaMalloc(&ctr, sizeof host);
    if (err == cudaSuccess) err = cudaMemsetAsync(ctr, 0, sizeof host, s);
    if (err == cudaSuccess) {
        if (h->fp32)
            launch_limiter(h->g, h->e, to_fields(q), h->cells32, h->fh32, h->gh32, h->fl32, h->gl32, h->theta32,
                           dt, nullptr, h->cnt, false, s, ctr);
        else
            launch_limiter(h->g, h->e, to_fields(q), Cells32{}, h->fh, h->gh, h->fl, h->gl, h->theta, dt, nullptr,
                           h->cnt, false, s, ctr);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(host, ctr, sizeof host, cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    cudaFree(ctr);
    if (err != cudaSuccess) {
        set_error("wm_verify_limiter_precheck", err);
        return WM_ERR_CUDA;
    }
    *decided = (long long)host[0];
    *disagreed = (long long)host[1];
    return WM_OK;
}

int wm_verify_switch_precheck(wm_handle *h, const wm_fields *q, long long *checked, long long *decided,
                              long long *disagreed, void *stream)
{
    if (!h || !fields_ok(h, q) || !checked || !decided || !disagreed) return WM_ERR_INVALID;
    unsigned long long *ctr = nullptr, host[3] = {0, 0, 0};
    cudaStream_t s = as_stream(stream);
    cudaError_t err = cudaMalloc(&ctr, sizeof host);
    if (err == cudaSuccess) err = cudaMemsetAsync(ctr, 0, sizeof host, s);
    if (err == cudaSuccess) {
        launch_verify_switch(h->g, h->e, to_fields(q), ctr, s);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(host, ctr, sizeof host, cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    cudaFree(ctr);
    if (err != cudaSuccess) {
        set_error("wm_verify_switch_precheck", err);
        return WM_ERR_CUDA;
    }
    *checked = (long long)host[0];
    *decided = (long long)host[1];
    *disagreed = (long long)host[2];
    return WM_OK;
}

int wm_verify_ducros_precheck(wm_handle *h, const wm_fields *q, long long *checked, long long *decided,
                              long long *disagreed, void *stream)
{
    if (!h || !fields_ok(h, q) || !checked || !decided || !disagreed) return WM_ERR_INVALID;
    unsigned long long *ctr = nullptr, host[3] = {0, 0, 0};
    cudaStream_t s = as_stream(stream);
    cudaError_t err = cudaMalloc(&ctr, sizeof host);
    if (err == cudaSuccess) err = cudaMemsetAsync(ctr, 0, sizeof host, s);
    if (err == cudaSuccess) {
        launch_verify_ducros(h->g, to_fields(q), ctr, s);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(host, ctr, sizeof host, cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    cudaFree(ctr);
    if (err != cudaSuccess) {
        set_error("wm_verify_ducros_precheck", err);
        return WM_ERR_CUDA;
    }
    *checked = (long long)host[0];
    *decided = (long long)host[1];
    *disagreed = (long long)host[2];
    return WM_OK;
}

int wm_set_prechecks(wm_handle *h, int on)
{
    if (!h) return WM_ERR_INVALID;
    if ((on != 0) != h->prechecks) drop_run_graph(h);
    h->prechecks = on != 0;
    return WM_OK;
}

int wm_set_limiter_sweeps(wm_handle *h, int in_place)
{
    if (!h) return WM_ERR_INVALID;
    const bool defer = in_place == 0;
    if (defer != h->defer_limiter) drop_run_graph(h);  // the captured loop used the other form
    h->defer_limiter = defer;
    return WM_OK;
}

int wm_read_workspace(wm_handle *h, int which, double *dst, void *stream)
{
    if (!h || !dst || which < 0 || which >= WM_WS_COUNT) return WM_ERR_INVALID;
    size_t n = (size_t)h->g.nxg * (size_t)h->g.nyg * sizeof(double);
    if (!h->arr[which]) {  // binary32 array of the precision form: widen into dst
        launch_widen(h->arr32[which], dst, (long long)h->g.nxg * h->g.nyg, as_stream(stream));
        return check_launch("wm_read_workspace");
    }
    cudaError_t err = cudaMemcpyAsync(dst, h->arr[which], n, cudaMemcpyDeviceToDevice, as_stream(stream));
    if (err != cudaSuccess) {
        set_error("wm_read_workspace", err);
        return WM_ERR_CUDA;
    }
    return WM_OK;
}

int wm_status(wm_handle *h, wm_stats *out, int reset, void *stream)
{
    if (!h || !out) return WM_ERR_INVALID;
    unsigned long long c[3];
    cudaStream_t s = as_stream(stream);
    cudaError_t err = cudaMemcpyAsync(c, h->ctr_base, sizeof c, cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess && reset) err = cudaMemsetAsync(h->ctr_base, 0, sizeof c, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) {
        set_error("wm_status", err);
        return WM_ERR_CUDA;
    }
    out->repaired_cells = (long long)c[0];
    out->nonfinite_cells = (long long)c[1];
    out->limited_cells = (long long)c[2];
    out->steps = h->steps;
    if (reset) h->steps = 0;
    return WM_OK;
}

int wm_probe_fp64_flops(double *flops, void *stream)
{
    if (!flops) return WM_ERR_INVALID;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    double *buf = nullptr;
    cudaError_t err = cudaMalloc(&buf, (size_t)blocks * threads * sizeof(double));
    if (err != cudaSuccess) {
        set_error("wm_probe_fp64_flops", err);
        return WM_ERR_NOMEM;
    }
    cudaStream_t s = as_stream(stream);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0, s);
        launch_fp64_probe(buf, iters, s, blocks, threads);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    int rc = check_launch("wm_probe_fp64_flops");
    if (rc) return rc;
    *flops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3);
    return WM_OK;
}

}  // extern "C"
