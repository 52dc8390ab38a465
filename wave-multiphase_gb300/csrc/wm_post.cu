// wm_post.cu -- schlieren post-processing on the device, the computation behind the reference's
// figure (save_png, SC:1728-1771) without a plotting library.
//
// grad[i*ny + j] = sqrt(drho/dx^2 + drho/dy^2) over the interior, rho = ar1 + ar2, with the
// derivatives taken by numpy.gradient's rule on the cell-centre coordinates (SC:1737-1739):
//   * inside, for unequal spacings h1 = x[i]-x[i-1], h2 = x[i+1]-x[i]:
//       a f[i-1] + b f[i] + c f[i+1],  a = -h2/(h1 (h1+h2)),  b = (h2-h1)/(h1 h2),  c = h1/(h2 (h1+h2));
//     when every spacing of the axis is the same number h: (f[i+1] - f[i-1]) / (2 h);
//   * at the two ends, first order: (f[1] - f[0]) / h and (f[n-1] - f[n-2]) / h.
// Every product and sum is rounded separately (no fused multiply-add) and the square root is the
// correctly rounded one, so the result equals numpy's bit for bit.
//
// The optional RGB image (ny rows, 2*nx columns, row r = y index j as the reference's imshow of
// the transposed array with origin 'upper' shows it) holds two panels: |grad rho| normalised to
// [1, 2400] through a nine-step blue ramp (ColorBrewer "Blues", the anchors of matplotlib's Blues),
// with the alpha1 = 0.5 level marked red where alpha1 - 0.5 changes sign towards the next cell in
// x or y; and alpha1 in inverted grey (0 white, 1 black).
#include <algorithm>
#include <cstdint>
#include <cstdio>

#include "../../include/wavemp.h"
#include "wm_device.cuh"

namespace wm {
void set_error_text(const char *msg);
}

namespace {

struct Axis {
    const double *h;  // n-1 spacings of the interior coordinates
    double h0;        // the common spacing when uniform
    int uniform;
    int n;
};

__device__ __forceinline__ double deriv(const double *f, long long stride, int i, const Axis &A)
{
    const int n = A.n;
    if (n < 2) return 0.0;
    if (i == 0) return __ddiv_rn(__dsub_rn(f[stride], f[0]), A.uniform ? A.h0 : A.h[0]);
    if (i == n - 1)
        return __ddiv_rn(__dsub_rn(f[0], f[-stride]), A.uniform ? A.h0 : A.h[n - 2]);
    if (A.uniform) return __ddiv_rn(__dsub_rn(f[stride], f[-stride]), __dmul_rn(2.0, A.h0));
    const double h1 = A.h[i - 1], h2 = A.h[i];
    const double s = __dadd_rn(h1, h2);
    const double a = __ddiv_rn(-h2, __dmul_rn(h1, s));
    const double b = __ddiv_rn(__dsub_rn(h2, h1), __dmul_rn(h1, h2));
    const double c = __ddiv_rn(h1, __dmul_rn(h2, s));
    return __dadd_rn(__dadd_rn(__dmul_rn(a, f[-stride]), __dmul_rn(b, f[0])), __dmul_rn(c, f[stride]));
}

// rho of the interior into a dense (nx, ny) scratch array (the derivative stencils read it)
__global__ void rho_kernel(const double *ar1, const double *ar2, long long pitch, int nx, int ny, int g,
                           double *rho)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (i >= nx || j >= ny) return;
    const long long k = (long long)(i + g) * pitch + (j + g);
    rho[(long long)i * ny + j] = __dadd_rn(ar1[k], ar2[k]);
}

__constant__ unsigned char kBlues[9][3] = {
    {0xf7, 0xfb, 0xff}, {0xde, 0xeb, 0xf7}, {0xc6, 0xdb, 0xef}, {0x9e, 0xca, 0xe1}, {0x6b, 0xae, 0xd6},
    {0x42, 0x92, 0xc6}, {0x21, 0x71, 0xb5}, {0x08, 0x51, 0x9c}, {0x08, 0x30, 0x6b}};

__global__ void grad_kernel(const double *rho, int nx, int ny, Axis X, Axis Y, const double *al,
                            long long pitch, int g, double *grad, unsigned char *rgb)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (i >= nx || j >= ny) return;
    const double *f = rho + (long long)i * ny + j;
    const double dx = deriv(f, ny, i, X), dy = deriv(f, 1, j, Y);
    const double m = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    grad[(long long)i * ny + j] = m;
    if (!rgb) return;
    const long long ka = (long long)(i + g) * pitch + (j + g);
    const double a = al[ka];
    unsigned char *px = rgb + ((long long)j * (2 * nx) + i) * 3;
    bool edge = false;
    if (i + 1 < nx) edge |= (a - 0.5) * (al[ka + pitch] - 0.5) < 0.0;
    if (j + 1 < ny) edge |= (a - 0.5) * (al[ka + 1] - 0.5) < 0.0;
    if (edge) {
        px[0] = 255;
        px[1] = 0;
        px[2] = 0;
    } else {
        double s = (m - 1.0) / (2400.0 - 1.0);
        s = s != s ? 0.0 : fmin(fmax(s, 0.0), 1.0);
        const double pos = s * 8.0;
        const int k0 = min((int)pos, 7);
        const double w = pos - k0;
        for (int c = 0; c < 3; ++c)
            px[c] = (unsigned char)lrint((1.0 - w) * kBlues[k0][c] + w * kBlues[k0 + 1][c]);
    }
    double v = a != a ? 0.0 : fmin(fmax(a, 0.0), 1.0);
    const unsigned char grey = (unsigned char)lrint(255.0 * (1.0 - v));
    unsigned char *pa = rgb + ((long long)j * (2 * nx) + nx + i) * 3;
    pa[0] = pa[1] = pa[2] = grey;
}

// to_f32 / to_f64 against the hardware conversions, bit for bit (NaN: both NaN).
__global__ void conv_check_kernel(const unsigned long long *in, long long n, unsigned long long *bad)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const double x = __longlong_as_double((long long)in[k]);
        const float a = wm::to_f32(x), b = __double2float_rn(x);
        const bool same32 = __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
        const float y = __uint_as_float((unsigned)in[k]);
        const double c = wm::to_f64(y), d = (double)y;
        const bool same64 = __double_as_longlong(c) == __double_as_longlong(d) || (c != c && d != d);
        // split32: hi is to_f32; lo the hardware rounding of x - hi (exact in binary64) in its
        // domain, 0 outside it
        float sh, sl;
        wm::split32(x, sh, sl);
        const int ex = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
        const bool dom = ex >= 949 && ex <= 1150 && !isinf(sh);
        const float lref = dom ? __double2float_rn(x - (double)sh) : 0.0f;
        const bool split_ok = __float_as_uint(sh) == __float_as_uint(a) &&
                              (dom ? __float_as_uint(sl) == __float_as_uint(lref) : (isinf(sh) || sl == 0.0f));
        if (!same32 || !split_ok) atomicAdd(&bad[0], 1ull);
        if (!same64) atomicAdd(&bad[1], 1ull);
        // integer binary64 compares against the hardware ones (pairs of neighbouring inputs)
        const double z = __longlong_as_double((long long)in[k + 1 < n ? k + 1 : 0]);
        const bool cmp_ok = wm::dlt(x, z) == (x < z) && wm::dlt(z, x) == (z < x) && wm::dneg(x) == (x < 0.0) &&
                            __double_as_longlong(wm::wmin(x, z)) == __double_as_longlong(x < z ? x : z) &&
                            __double_as_longlong(wm::wmax(x, z)) == __double_as_longlong(x > z ? x : z) &&
                            wm::wsign(x) == (x < 0.0 ? -1.0 : 1.0) && wm::dle(x, z) == (x <= z) &&
                            wm::dle(z, x) == (z <= x) && wm::dpos(x) == (x > 0.0) &&
                            wm::wisnan(x) == (x != x);
        if (!cmp_ok) atomicAdd(&bad[2], 1ull);
    }
}

// One result of the sweep's arithmetic against the IEEE one: 0 same bits, 1 one unit in the last
// place apart (both finite, normal and of one sign), 2 otherwise (NaN: both NaN counts as same).
__device__ int ulp_class(double a, double b)
{
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    if (ia == ib || (a != a && b != b)) return 0;
    const long long ma = ia & 0x7fffffffffffffffLL, mb = ib & 0x7fffffffffffffffLL;
    const long long lo = 0x0010000000000000LL, hi = 0x7ff0000000000000LL;  // normal range
    if ((ia ^ ib) < 0 || ma < lo || mb < lo || ma >= hi || mb >= hi) return 2;
    return (ma - mb == 1 || mb - ma == 1) ? 1 : 2;
}

// The reference's minmod products on the hardware binary64 operations (the generic mm2 / mm4).
__device__ double mm2_hw(double x, double y)
{
    const double sx = x < 0.0 ? -1.0 : 1.0, sy = y < 0.0 ? -1.0 : 1.0, ax = fabs(x), ay = fabs(y);
    return __dmul_rn(__dmul_rn(0.5, __dadd_rn(sx, sy)), ax < ay ? ax : ay);
}
__device__ double mm4_hw(double a, double b, double c, double d)
{
    const double sa = a < 0.0 ? -1.0 : 1.0, sb = b < 0.0 ? -1.0 : 1.0;
    const double sc = c < 0.0 ? -1.0 : 1.0, sd = d < 0.0 ? -1.0 : 1.0;
    const double m1 = fabs(a) < fabs(b) ? fabs(a) : fabs(b), m2 = fabs(c) < fabs(d) ? fabs(c) : fabs(d);
    const double p = fabs(__dmul_rn(__dadd_rn(sa, sc), __dadd_rn(sa, sd)));
    return __dmul_rn(__dmul_rn(__dmul_rn(0.125, __dadd_rn(sa, sb)), p), m1 < m2 ? m1 : m2);
}
__device__ bool same_bits(double a, double b)
{
    return __double_as_longlong(a) == __double_as_longlong(b) || (a != a && b != b);
}
// a within n units in the last place of b (both finite, normal and of one sign), or the same bits
__device__ bool within_ulps(double a, double b, long long n)
{
    if (same_bits(a, b)) return true;
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const long long ma = ia & 0x7fffffffffffffffLL, mb = ib & 0x7fffffffffffffffLL;
    const long long lo = 0x0010000000000000LL, hi = 0x7ff0000000000000LL;
    if ((ia ^ ib) < 0 || ma < lo || mb < lo || ma >= hi || mb >= hi) return false;
    return ma - mb <= n && mb - ma <= n;
}

__global__ void sweep_arith_kernel(const unsigned long long *in, long long n, unsigned long long *cnt)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const double y = __longlong_as_double((long long)in[k]);
        const double x = __longlong_as_double((long long)in[(k + 1) % n]);
        const double z = __longlong_as_double((long long)in[(k + 2) % n]);
        const double w = __longlong_as_double((long long)in[(k + 3) % n]);
        const int c[3] = {ulp_class(wm::rcp_nr(y), 1.0 / y), ulp_class(wm::div_nr(x, y), x / y),
                          ulp_class(wm::sqrt_nr(fabs(y)), sqrt(fabs(y)))};
        for (int t = 0; t < 3; ++t)
            if (c[t]) atomicAdd(&cnt[c[t] == 2 ? t : 3 + t], 1ull);
        if (!same_bits(wm::mm2(y, x), mm2_hw(y, x))) atomicAdd(&cnt[6], 1ull);
        if (!same_bits(wm::mm4(y, x, z, w), mm4_hw(y, x, z, w))) atomicAdd(&cnt[7], 1ull);
        if (!same_bits(wm::half_of(y), __dmul_rn(0.5, y))) atomicAdd(&cnt[8], 1ull);
        const double s = (k & 1) ? -1.0 : 1.0;
        const double sel = __fma_rn(__dmul_rn(0.5, __dadd_rn(1.0, s)), y, __dmul_rn(__dmul_rn(0.5, __dadd_rn(1.0, -s)), x));
        if (!same_bits(wm::sign_select(s, y, x), sel)) atomicAdd(&cnt[9], 1ull);
        double q1, q2;
        wm::div2_nr(x, y, w, z, q1, q2);
        if (!within_ulps(q1, x / y, 4) || !within_ulps(q2, w / z, 4)) atomicAdd(&cnt[10], 1ull);
    }
}

}  // namespace

extern "C" int wm_check_sweep_arith(const unsigned long long *bits, long long n, long long counts[11], void *stream)
{
    if (!bits || n < 0 || !counts) return WM_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned long long *ctr = nullptr, host[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    cudaError_t e = cudaMalloc(&ctr, sizeof host);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctr, 0, sizeof host, s);
    if (e == cudaSuccess && n > 0) {
        sweep_arith_kernel<<<1024, 256, 0, s>>>(bits, n, ctr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, ctr, sizeof host, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(ctr);
    if (e != cudaSuccess) {
        char msg[200];
        snprintf(msg, sizeof msg, "wm_check_sweep_arith: %s", cudaGetErrorString(e));
        wm::set_error_text(msg);
        return WM_ERR_CUDA;
    }
    for (int t = 0; t < 11; ++t) counts[t] = (long long)host[t];
    return WM_OK;
}

extern "C" int wm_check_conversions(const unsigned long long *bits, long long n, long long *bad_f32,
                                    long long *bad_f64, long long *bad_cmp, void *stream)
{
    if (!bits || n < 0 || !bad_f32 || !bad_f64 || !bad_cmp) return WM_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned long long *ctr = nullptr, host[3] = {0, 0, 0};
    cudaError_t e = cudaMalloc(&ctr, sizeof host);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctr, 0, sizeof host, s);
    if (e == cudaSuccess && n > 0) {
        conv_check_kernel<<<1024, 256, 0, s>>>(bits, n, ctr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, ctr, sizeof host, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(ctr);
    if (e != cudaSuccess) {
        char msg[200];
        snprintf(msg, sizeof msg, "wm_check_conversions: %s", cudaGetErrorString(e));
        wm::set_error_text(msg);
        return WM_ERR_CUDA;
    }
    *bad_f32 = (long long)host[0];
    *bad_f64 = (long long)host[1];
    *bad_cmp = (long long)host[2];
    return WM_OK;
}

extern "C" int wm_schlieren(const wm_fields *q, int nx, int ny, int g, const double *xh, const double *yh,
                            double x_h0, double y_h0, double *rho_scratch, double *grad,
                            unsigned char *rgb, void *stream)
{
    if (!q || !q->ar1 || !q->ar2 || !q->al || !rho_scratch || !grad || nx < 2 || ny < 2 || nx > 65535 || g < 0 ||
        q->pitch < ny + 2 * g || (!xh && !(x_h0 != 0.0)) || (!yh && !(y_h0 != 0.0)))
        return WM_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const dim3 block(128), grid((ny + 127) / 128, nx);
    rho_kernel<<<grid, block, 0, s>>>(q->ar1, q->ar2, q->pitch, nx, ny, g, rho_scratch);
    const Axis X{xh, x_h0, xh == nullptr, nx}, Y{yh, y_h0, yh == nullptr, ny};
    grad_kernel<<<grid, block, 0, s>>>(rho_scratch, nx, ny, X, Y, q->al, q->pitch, g, grad, rgb);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        char msg[200];
        snprintf(msg, sizeof msg, "wm_schlieren: %s", cudaGetErrorString(e));
        wm::set_error_text(msg);
        return WM_ERR_CUDA;
    }
    return WM_OK;
}

namespace {

// n 16-byte words from src to dst by the SMs, four loads in flight per thread before its stores
// (latency of a host-side operand read over the chip-to-chip link hidden by the loads in flight).
__global__ void __launch_bounds__(256) state_copy_kernel(uint4 *__restrict__ dst, const uint4 *__restrict__ src,
                                                         long long n)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; k + 3 * stride < n; k += 4 * stride) {
        const uint4 a = src[k], b = src[k + stride], c = src[k + 2 * stride], d = src[k + 3 * stride];
        dst[k] = a;
        dst[k + stride] = b;
        dst[k + 2 * stride] = c;
        dst[k + 3 * stride] = d;
    }
    for (; k < n; k += stride) dst[k] = src[k];
}

// The address a kernel on device `dev` uses for p: p itself for managed memory and for device memory
// of `dev`, the mapped address of page-locked host memory; nullptr for memory that device cannot
// address that way (another device's memory included). `kind` receives the memory type.
const char *device_view(const void *p, int dev, int &kind)
{
    cudaPointerAttributes a;
    kind = -1;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    kind = (int)a.type;
    if (a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev))
        return static_cast<const char *>(p);
    if (a.type == cudaMemoryTypeHost) {
        void *d = nullptr;
        if (cudaHostGetDevicePointer(&d, const_cast<void *>(p), 0) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return static_cast<const char *>(d);
    }
    return nullptr;
}

// Device view of the range [p, p + bytes): both ends in memory of the same kind that maps to one
// contiguous device range, else nullptr. The ends only: a range that runs past its allocation into
// an adjacent one of the same kind is not detected.
const char *range_view(const void *p, long long bytes, int dev)
{
    int k0, k1;
    const char *d0 = device_view(p, dev, k0);
    const char *d1 = device_view(static_cast<const char *>(p) + (bytes - 1), dev, k1);
    if (!d0 || !d1 || k0 != k1 || d1 - d0 != bytes - 1) return nullptr;
    return d0;
}

}  // namespace

extern "C" int wm_copy_state(void *dst, const void *src, long long bytes, void *stream)
{
    if (!dst || !src || bytes < 0 || bytes % 16 != 0 || (reinterpret_cast<uintptr_t>(dst) & 15) ||
        (reinterpret_cast<uintptr_t>(src) & 15)) {
        wm::set_error_text("wm_copy_state: addresses must be 16-byte aligned and bytes a multiple of 16");
        return WM_ERR_INVALID;
    }
    if (bytes == 0) return WM_OK;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        wm::set_error_text("wm_copy_state: no CUDA device");
        return WM_ERR_CUDA;
    }
    const char *d = range_view(dst, bytes, dev), *s = range_view(src, bytes, dev);
    if (!d || !s) {
        wm::set_error_text("wm_copy_state: a buffer is neither memory of the current device nor page-locked "
                           "host memory mapped for it over its whole range");
        return WM_ERR_INVALID;
    }
    const long long n = bytes / 16;
    // 4 resident blocks of 256 a SM (64 registers): one wave, four 16-byte loads in flight a thread
    const long long blocks = std::min<long long>((n + 255) / 256, 4LL * sms);
    state_copy_kernel<<<(unsigned)blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<uint4 *>(const_cast<char *>(d)), reinterpret_cast<const uint4 *>(s), n);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        char msg[200];
        snprintf(msg, sizeof msg, "wm_copy_state: %s", cudaGetErrorString(e));
        wm::set_error_text(msg);
        return WM_ERR_CUDA;
    }
    return WM_OK;
}
