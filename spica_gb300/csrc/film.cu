// film.cu -- the film output path on the device: Film::save's resolve of the
// accumulated film (core/film.cc:23-30), the reference's RGBE encoding of an HDR image
// (HDRPixel, core/image.cc:63-99) and its tone-mapping operators (GammaTmo, ReinhardTmo,
// DragoTmo, DurandTMO, core/tmo.cc:53-243, with Image::toByte, core/image.cc:476, and the
// bilateral filter of core/birateral.cc),
// plus host writers for the reference's .hdr file layout (Image::saveHdr,
// core/image.cc:390-434) and a minimal PNG.
//
// The per-pixel arithmetic is FP64, in the reference's order, so that the encoded
// bytes equal the reference's for the same float film.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_reduce.cuh>

#include "../../include/spica_gpu.h"
#include "ctx.cuh"

namespace spgpu {

namespace {

constexpr double kRefEps = 1.0e-12;   // EPS, core/common.h:55

// Film::save: pixel / (weight + EPS), per channel (core/film.cc:25-28)
__device__ __forceinline__ void resolvePixel(const float4 f, double *r, double *g, double *b) {
    const double w = static_cast<double>(f.w) + kRefEps;
    *r = static_cast<double>(f.x) / w;
    *g = static_cast<double>(f.y) / w;
    *b = static_cast<double>(f.z) / w;
}

__host__ __device__ __forceinline__ double gray(double r, double g, double b) {   // RGBSpectrum::gray
    return 0.2126 * r + 0.7152 * g + 0.0722 * b;
}

// HDRPixel(color): shared exponent of the largest channel (core/image.cc:72-88)
__host__ __device__ __forceinline__ void rgbeEncode(double r, double g, double b, uint8_t *out) {
    double d = r > g ? r : g;
    d = d > b ? d : b;
    if (d <= 1.0e-32) {
        out[0] = out[1] = out[2] = out[3] = 0;
        return;
    }
    int ie;
    const double m = frexp(d, &ie);
    d = m * 256.0 / d;
    out[0] = static_cast<uint8_t>(r * d);
    out[1] = static_cast<uint8_t>(g * d);
    out[2] = static_cast<uint8_t>(b * d);
    out[3] = static_cast<uint8_t>(ie + 128);
}

// Image::toByte (core/image.cc:476)
__device__ __forceinline__ uint8_t toByte(double d) {
    d = fmax(0.0, fmin(d, 1.0));
    return static_cast<uint8_t>(255.0 * d);
}

__global__ void k_film_rgbe(const float4 *__restrict__ film, int n, uint8_t *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r, g, b;
        resolvePixel(film[i], &r, &g, &b);
        uint8_t e[4];
        rgbeEncode(r, g, b, e);
        reinterpret_cast<uchar4 *>(out)[i] = make_uchar4(e[0], e[1], e[2], e[3]);
    }
}

// GammaTmo::apply then Image::toByte, as LDRFilm::saveImage (films/ldrfilm.cc:25-31)
__global__ void k_film_gamma(const float4 *__restrict__ film, int n, double invG, uint8_t *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r, g, b;
        resolvePixel(film[i], &r, &g, &b);
        out[3 * static_cast<int64_t>(i) + 0] = toByte(fmin(fmax(pow(r, invG), 0.0), 1.0));
        out[3 * static_cast<int64_t>(i) + 1] = toByte(fmin(fmax(pow(g, invG), 0.0), 1.0));
        out[3 * static_cast<int64_t>(i) + 2] = toByte(fmin(fmax(pow(b, invG), 0.0), 1.0));
    }
}

// luminance of each resolved pixel, and the sum of log(L + EPS) (logMean, core/tmo.cc:15)
__global__ void k_film_gray(const float4 *__restrict__ film, int n, double *grayOut, double *logSum) {
    double part = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r, g, b;
        resolvePixel(film[i], &r, &g, &b);
        const double L = gray(r, g, b);
        grayOut[i] = L;
        part += log(L + kRefEps);
    }
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(logSum, part);
}

// ReinhardTmo::apply (core/tmo.cc:81-101); lw[0] = log sum, lw[1] / lw[2] = sorted
// luminances at the white point's two order statistics
__global__ void k_film_reinhard(const float4 *__restrict__ film, int n, double alpha, const double *lw,
                                const double *lmin, const double *lmax, float *out) {
    const double Lwa = exp(lw[0] / n);
    const double log2Max = log2(*lmax + kRefEps), log2Min = log2(*lmin + kRefEps);
    const double Lwhite = 1.5 * pow(2.0, log2Max - log2Min - 5);   // ReinhardTmo::whitePoint, tmo.cc:123
    const double Lwhite2 = Lwhite * Lwhite;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r, g, b;
        resolvePixel(film[i], &r, &g, &b);
        const double L = gray(r, g, b);
        const double Ls = (alpha * L) / Lwa;
        const double Ld = (Ls * (1.0 + Ls / Lwhite2)) / (1.0 + Ls);
        const double s = L + kRefEps;
        out[3 * static_cast<int64_t>(i) + 0] = static_cast<float>(r / s * Ld);
        out[3 * static_cast<int64_t>(i) + 1] = static_cast<float>(g / s * Ld);
        out[3 * static_cast<int64_t>(i) + 2] = static_cast<float>(b / s * Ld);
    }
}

// gray() of an RGB spectrum whose three channels hold v (the reference stores luminances
// that way and reads them back with gray(), which is not always v)
__host__ __device__ __forceinline__ double grayRep(double v) { return 0.2126 * v + 0.7152 * v + 0.0722 * v; }

// DragoTmo::apply with Ldmax 100 (core/tmo.cc:135-159); lw = log sum, lmax = the largest
// luminance (lumMax, starting from 0)
__global__ void k_film_drago(const float4 *__restrict__ film, int n, double p, const double *lw, const double *lmax,
                             float *out) {
    const double Lwa = exp(lw[0] / n) / pow(1.0 + p - 0.85, 5.0);
    const double Lmax_wa = fmax(0.0, *lmax) / Lwa;
    const double c1 = log(p) / log(0.5);
    const double c2 = (100.0 / 100.0) / log10(1.0 + Lmax_wa);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r, g, b;
        resolvePixel(film[i], &r, &g, &b);
        const double L = gray(r, g, b);
        const double L_wa = L / Lwa;
        const double Ld = c2 * log1p(L_wa) / log(2.0 + 8.0 * pow(L_wa / Lmax_wa, c1));
        const double s = L + kRefEps;
        out[3 * static_cast<int64_t>(i) + 0] = static_cast<float>(r / s * Ld);
        out[3 * static_cast<int64_t>(i) + 1] = static_cast<float>(g / s * Ld);
        out[3 * static_cast<int64_t>(i) + 2] = static_cast<float>(b / s * Ld);
    }
}

// DurandTMO (core/tmo.cc:171-243) with the reference's bilateral filter, the recursive
// domain-transform filter of Gastal and Oliveira (core/birateral.cc): luminances l, the
// filter's input log10(gray(l) + 1e-6), and the transformed-domain derivatives
// dctx[y][x] = 1 + (sigma_s / sigma_r) |dI/dx| (W-1 per row), dcty[y][x] likewise (H-1 rows)
__global__ void k_durand_prepare(const float4 *__restrict__ film, int n, double *lum, double *logL) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r, g, b;
        resolvePixel(film[i], &r, &g, &b);
        const double l = gray(r, g, b);
        lum[i] = l;
        logL[i] = log10(grayRep(l) + 1.0e-6);
    }
}
__global__ void k_durand_dct(const double *__restrict__ logL, int W, int H, double ratio, double *dctx,
                             double *dcty) {
    const int n = W * H;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int y = i / W, x = i - y * W;
        if (x < W - 1) dctx[static_cast<int64_t>(y) * (W - 1) + x] = 1.0 + ratio * fabs(logL[i + 1] - logL[i]);
        if (y < H - 1) dcty[i] = 1.0 + ratio * fabs(logL[i + W] - logL[i]);
    }
}
// the feedback coefficients of one iteration, a^dct for both directions (the V tables of
// recursiveFilterHorizontal / recursiveFilterVertical), all pixels in parallel so that the
// line scans below carry no pow on their serial chain
__global__ void k_durand_pow(const double *__restrict__ dct, int64_t m, double a, double *V) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < m;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        V[i] = pow(a, dct[i]);
}
// one horizontal pass (recursiveFilterHorizontal): per row, forward then backward; the
// update keeps the reference's rounding (no contraction into an fma)
__global__ void k_durand_rows(double *f, const double *__restrict__ Vx, int W, int H) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= H) return;
    double *row = f + static_cast<int64_t>(y) * W;
    const double *p = Vx + static_cast<int64_t>(y) * (W - 1);
    double prev = row[0];
    for (int x = 1; x < W; x++) {
        prev = __dadd_rn(row[x], __dmul_rn(p[x - 1], prev - row[x]));
        row[x] = prev;
    }
    for (int x = W - 2; x >= 0; x--) {
        prev = __dadd_rn(row[x], __dmul_rn(p[x], prev - row[x]));
        row[x] = prev;
    }
}
// one vertical pass (recursiveFilterVertical): per column, forward then backward
__global__ void k_durand_cols(double *f, const double *__restrict__ Vy, int W, int H) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    double prev = f[x];
    for (int y = 1; y < H; y++) {
        double &v = f[static_cast<int64_t>(y) * W + x];
        prev = __dadd_rn(v, __dmul_rn(Vy[static_cast<int64_t>(y - 1) * W + x], prev - v));
        v = prev;
    }
    for (int y = H - 2; y >= 0; y--) {
        double &v = f[static_cast<int64_t>(y) * W + x];
        prev = __dadd_rn(v, __dmul_rn(Vy[static_cast<int64_t>(y) * W + x], prev - v));
        v = prev;
    }
}
// base and detail layers (birateralSeparation), their logarithms (DurandTMO::apply)
__global__ void k_durand_layers(const double *__restrict__ lum, const double *__restrict__ filt, int n,
                                double *logBase, double *logDetail) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double lb = fmax(0.0, pow(10.0, grayRep(filt[i])) - 1.0e-6);
        const double ld = lum[i] / (lb + kRefEps);
        logBase[i] = log10(grayRep(lb) + kRefEps);
        logDetail[i] = log10(grayRep(ld) + kRefEps);
    }
}
__global__ void k_durand_apply(const float4 *__restrict__ film, const double *__restrict__ lum,
                               const double *__restrict__ logBase, const double *__restrict__ logDetail, int n,
                               double contrast, const double *maxLog, const double *minLog, float *out) {
    const double cf = log(contrast) / (*maxLog - *minLog);
    const double logAbs = cf * *maxLog;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r, g, b;
        resolvePixel(film[i], &r, &g, &b);
        const double s = lum[i] + kRefEps;
        const double m = pow(10.0, grayRep(logBase[i]) * cf + grayRep(logDetail[i]) - logAbs);
        out[3 * static_cast<int64_t>(i) + 0] = static_cast<float>(fmin(fmax(r / s * m, 0.0), 1.0));
        out[3 * static_cast<int64_t>(i) + 1] = static_cast<float>(fmin(fmax(g / s * m, 0.0), 1.0));
        out[3 * static_cast<int64_t>(i) + 2] = static_cast<float>(fmin(fmax(b / s * m, 0.0), 1.0));
    }
}

int launchGrid(int n) { return std::max(1, std::min((n + 255) / 256, 152 * 8)); }

// ---------------------------------------------------------------- host writers
uint32_t crc32Table[256];
bool crcInit = false;
uint32_t crc32(const uint8_t *p, size_t n, uint32_t c = 0xFFFFFFFFu) {
    if (!crcInit) {   // the PNG specification's CRC-32 (polynomial 0xEDB88320)
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t v = i;
            for (int k = 0; k < 8; k++) v = (v & 1u) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
            crc32Table[i] = v;
        }
        crcInit = true;
    }
    for (size_t i = 0; i < n; i++) c = crc32Table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
    return c;
}
void put32(std::vector<uint8_t> &v, uint32_t x) {
    v.push_back(static_cast<uint8_t>(x >> 24));
    v.push_back(static_cast<uint8_t>(x >> 16));
    v.push_back(static_cast<uint8_t>(x >> 8));
    v.push_back(static_cast<uint8_t>(x));
}
void pngChunk(std::vector<uint8_t> &file, const char *type, const std::vector<uint8_t> &data) {
    put32(file, static_cast<uint32_t>(data.size()));
    const size_t start = file.size();
    file.insert(file.end(), type, type + 4);
    file.insert(file.end(), data.begin(), data.end());
    put32(file, crc32(file.data() + start, file.size() - start) ^ 0xFFFFFFFFu);
}

}  // namespace

int filmResolve(Ctx &C, const float *film, int W, int H, int format, double param, void *out, cudaStream_t s) {
    const int n = W * H;
    const float4 *f4 = reinterpret_cast<const float4 *>(film);
    cudaError_t e = cudaSuccess;
    if (format == SPGPU_FILM_RGBE) {
        k_film_rgbe<<<launchGrid(n), 256, 0, s>>>(f4, n, static_cast<uint8_t *>(out));
        e = cudaGetLastError();
    } else if (format == SPGPU_FILM_GAMMA_BYTES) {
        k_film_gamma<<<launchGrid(n), 256, 0, s>>>(f4, n, 1.0 / param, static_cast<uint8_t *>(out));
        e = cudaGetLastError();
    } else if (format == SPGPU_FILM_DRAGO) {   // luminances, their log mean and maximum
        const double p = param > 0.0 ? param : 0.85;
        double *buf = nullptr;
        void *tmp = nullptr;
        size_t tmpBytes = 0;
        cub::DeviceReduce::Max(nullptr, tmpBytes, static_cast<const double *>(nullptr), static_cast<double *>(nullptr),
                               n, s);
        e = cudaMallocAsync(&buf, sizeof(double) * (static_cast<size_t>(n) + 2), s);
        if (e == cudaSuccess) e = cudaMallocAsync(&tmp, std::max<size_t>(tmpBytes, 16), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(buf + n, 0, sizeof(double), s);
        if (e == cudaSuccess) {
            k_film_gray<<<launchGrid(n), 256, 0, s>>>(f4, n, buf, buf + n);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cub::DeviceReduce::Max(tmp, tmpBytes, buf, buf + n + 1, n, s);
        if (e == cudaSuccess) {
            k_film_drago<<<launchGrid(n), 256, 0, s>>>(f4, n, p, buf + n, buf + n + 1, static_cast<float *>(out));
            e = cudaGetLastError();
        }
        if (buf) cudaFreeAsync(buf, s);
        if (tmp) cudaFreeAsync(tmp, s);
    } else if (format == SPGPU_FILM_DURAND) {
        const double contrast = param > 0.0 ? param : 5.0;
        const int maxiter = 20;
        const double sigmaS = std::max(W, H) * 0.02, sigmaR = 0.4;   // DurandTMO defaults, tmo.h:74
        const size_t N = static_cast<size_t>(n);
        double *buf = nullptr;   // lum | filtered | dctx | dcty | logBase | logDetail | Vx | Vy | max | min
        void *tmp = nullptr;
        size_t t1 = 0, t2 = 0;
        cub::DeviceReduce::Max(nullptr, t1, static_cast<const double *>(nullptr), static_cast<double *>(nullptr), n, s);
        cub::DeviceReduce::Min(nullptr, t2, static_cast<const double *>(nullptr), static_cast<double *>(nullptr), n, s);
        const size_t tmpBytes = std::max<size_t>(std::max(t1, t2), 16);
        e = cudaMallocAsync(&buf, sizeof(double) * (8 * N + 2), s);
        if (e == cudaSuccess) e = cudaMallocAsync(&tmp, tmpBytes, s);
        double *lum = buf, *filt = buf + N, *dctx = buf + 2 * N, *dcty = buf + 3 * N, *logBase = buf + 4 * N,
               *logDetail = buf + 5 * N, *Vx = buf + 6 * N, *Vy = buf + 7 * N, *mx = buf + 8 * N, *mn = mx + 1;
        const int64_t nx = static_cast<int64_t>(H) * (W - 1), ny = static_cast<int64_t>(H - 1) * W;
        if (e == cudaSuccess) {
            k_durand_prepare<<<launchGrid(n), 256, 0, s>>>(f4, n, lum, filt);
            k_durand_dct<<<launchGrid(n), 256, 0, s>>>(filt, W, H, sigmaS / sigmaR, dctx, dcty);
            for (int i = 0; i < maxiter; i++) {   // domainTransformFilter, birateral.cc:118-122
                const double sigmaH =
                    sigmaS * std::sqrt(3.0) * std::pow(2.0, maxiter - i - 1) / std::sqrt(std::pow(4.0, maxiter) - 1.0);
                const double a = std::exp(-std::sqrt(2.0) / sigmaH);
                if (nx > 0) k_durand_pow<<<launchGrid(static_cast<int>(nx)), 256, 0, s>>>(dctx, nx, a, Vx);
                if (ny > 0) k_durand_pow<<<launchGrid(static_cast<int>(ny)), 256, 0, s>>>(dcty, ny, a, Vy);
                k_durand_rows<<<(H + 127) / 128, 128, 0, s>>>(filt, Vx, W, H);
                k_durand_cols<<<(W + 127) / 128, 128, 0, s>>>(filt, Vy, W, H);
            }
            k_durand_layers<<<launchGrid(n), 256, 0, s>>>(lum, filt, n, logBase, logDetail);
            e = cudaGetLastError();
        }
        size_t tb = tmpBytes;
        if (e == cudaSuccess) e = cub::DeviceReduce::Max(tmp, tb, logBase, mx, n, s);
        tb = tmpBytes;
        if (e == cudaSuccess) e = cub::DeviceReduce::Min(tmp, tb, logBase, mn, n, s);
        if (e == cudaSuccess) {
            k_durand_apply<<<launchGrid(n), 256, 0, s>>>(f4, lum, logBase, logDetail, n, contrast, mx, mn,
                                                          static_cast<float *>(out));
            e = cudaGetLastError();
        }
        if (buf) cudaFreeAsync(buf, s);
        if (tmp) cudaFreeAsync(tmp, s);
    } else {   // SPGPU_FILM_REINHARD: luminances, their log mean and two order statistics
        double *buf = nullptr;
        void *tmp = nullptr;
        size_t tmpBytes = 0;
        cub::DeviceRadixSort::SortKeys(nullptr, tmpBytes, static_cast<const double *>(nullptr),
                                       static_cast<double *>(nullptr), n, 0, 64, s);
        e = cudaMallocAsync(&buf, sizeof(double) * (2 * static_cast<size_t>(n) + 1), s);
        if (e == cudaSuccess) e = cudaMallocAsync(&tmp, std::max<size_t>(tmpBytes, 16), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(buf + 2 * static_cast<size_t>(n), 0, sizeof(double), s);
        if (e == cudaSuccess) {
            k_film_gray<<<launchGrid(n), 256, 0, s>>>(f4, n, buf, buf + 2 * static_cast<size_t>(n));
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cub::DeviceRadixSort::SortKeys(tmp, tmpBytes, buf, buf + n, n, 0, 64, s);
        // ReinhardTmo::whitePoint's indices (tmo.cc:118-119)
        const int iMax = std::min(static_cast<int>(n * 0.99), n - 1);
        const int iMin = std::min(static_cast<int>(n * 0.01), n - 1);
        if (e == cudaSuccess) {
            k_film_reinhard<<<launchGrid(n), 256, 0, s>>>(f4, n, param, buf + 2 * static_cast<size_t>(n),
                                                           buf + n + iMin, buf + n + iMax, static_cast<float *>(out));
            e = cudaGetLastError();
        }
        if (buf) cudaFreeAsync(buf, s);
        if (tmp) cudaFreeAsync(tmp, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? 0 : cudaFail("spgpu_film_resolve", e);
}

// Image::saveHdr's header and scanlines: per row the new-style RLE marker (2, 2, width)
// and each of the four channels as literal runs of at most 127 bytes
int writeHdr(const char *path, const uint8_t *rgbe, int W, int H) {
    std::vector<uint8_t> file;
    const char nl = 0x0a;
    char buf[256];
    const std::string header = std::string("#?RADIANCE") + nl + "# Made with 100% pure HDR Shop" + nl +
                               "FORMAT=32-bit_rle_rgbe" + nl + "EXPOSURE=1.0000000000000" + nl + nl;
    file.insert(file.end(), header.begin(), header.end());
    std::snprintf(buf, sizeof(buf), "-Y %u +X %u%c", static_cast<unsigned>(H), static_cast<unsigned>(W), nl);
    file.insert(file.end(), buf, buf + std::strlen(buf));
    const unsigned w = static_cast<unsigned>(W);
    for (int y = 0; y < H; y++) {
        const uint8_t *row = rgbe + 4 * static_cast<size_t>(y) * W;
        file.push_back(0x02);
        file.push_back(0x02);
        file.push_back(static_cast<uint8_t>((w >> 8) & 0xFFu));
        file.push_back(static_cast<uint8_t>(w & 0xFFu));
        for (int c = 0; c < 4; c++) {
            for (unsigned cursor = 0; cursor < w;) {
                const unsigned run = std::min(127u, w - cursor);
                file.push_back(static_cast<uint8_t>(run));
                for (unsigned j = cursor; j < cursor + run; j++) file.push_back(row[4 * j + c]);
                cursor += run;
            }
        }
    }
    FILE *fp = std::fopen(path, "wb");
    if (!fp) {
        setError(std::string("spgpu_write_hdr: cannot open ") + path);
        return SPGPU_EINVAL;
    }
    const size_t wrote = std::fwrite(file.data(), 1, file.size(), fp);
    std::fclose(fp);
    if (wrote != file.size()) {
        setError(std::string("spgpu_write_hdr: short write to ") + path);
        return SPGPU_EINVAL;
    }
    return 0;
}

// 8-bit RGB PNG: zlib stream of stored (uncompressed) deflate blocks, filter 0 per row
int writePng(const char *path, const uint8_t *rgb, int W, int H) {
    std::vector<uint8_t> raw;
    raw.reserve(static_cast<size_t>(H) * (3 * W + 1));
    for (int y = 0; y < H; y++) {
        raw.push_back(0);
        raw.insert(raw.end(), rgb + 3 * static_cast<size_t>(y) * W, rgb + 3 * static_cast<size_t>(y + 1) * W);
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    uint32_t a = 1, b = 0;   // Adler-32
    for (uint8_t v : raw) {
        a = (a + v) % 65521u;
        b = (b + a) % 65521u;
    }
    for (size_t off = 0; off < raw.size() || off == 0;) {
        const size_t len = std::min<size_t>(65535, raw.size() - off);
        const bool last = off + len >= raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back(static_cast<uint8_t>(len & 0xFF));
        z.push_back(static_cast<uint8_t>(len >> 8));
        z.push_back(static_cast<uint8_t>(~len & 0xFF));
        z.push_back(static_cast<uint8_t>((~len >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
        off += len;
        if (last) break;
    }
    put32(z, (b << 16) | a);
    std::vector<uint8_t> file = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    std::vector<uint8_t> ihdr;
    put32(ihdr, static_cast<uint32_t>(W));
    put32(ihdr, static_cast<uint32_t>(H));
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});   // 8-bit, truecolour, deflate, filter 0, no interlace
    pngChunk(file, "IHDR", ihdr);
    pngChunk(file, "IDAT", z);
    pngChunk(file, "IEND", {});
    FILE *fp = std::fopen(path, "wb");
    if (!fp) {
        setError(std::string("spgpu_write_png: cannot open ") + path);
        return SPGPU_EINVAL;
    }
    const size_t wrote = std::fwrite(file.data(), 1, file.size(), fp);
    std::fclose(fp);
    if (wrote != file.size()) {
        setError(std::string("spgpu_write_png: short write to ") + path);
        return SPGPU_EINVAL;
    }
    return 0;
}

}  // namespace spgpu
