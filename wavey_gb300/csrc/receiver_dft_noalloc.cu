// receiver_dft_noalloc.cu -- the receiver DFT without any device allocation.
//
// Some callers cannot allocate device memory when they want the spectra:
// a real-time audio host calling from its processing thread (cudaMalloc and
// cudaFree may synchronise the whole device and take milliseconds, which
// breaks an audio deadline), or an application whose device memory is
// entirely owned by its own pool allocator and forbids other allocations.
// For them, wavey_cuda_receiver_dft_noalloc turns receiver time series that
// are already on the device into FP64 spectra with the same chunked
// algorithm as the FDTD runs (FP32 sums over 128-step chunks against
// exp(-j 2 pi frac(f dt n)) twiddles, added into FP64), using only memory the
// caller passes in plus one fixed scratch array compiled into this library.
//
// The scratch is g_noalloc_twiddles below: 128 steps x 2048 frequencies of
// FP32 complex twiddles, 2 MiB, held by every GPU that loads this library
// until the process exits.  Host code never uses the symbol itself as a
// pointer (on the host it is only a stand-in for the device variable): the
// first call on each device looks up its device address with
// cudaGetSymbolAddress while that device is current, and passes that address
// to the kernels.  That first call should therefore be made before any
// stream capture begins.
//
// Every call shares the one scratch array, and each call overwrites it
// completely before reading it, so nothing in it needs clearing; the output
// is cleared by the call itself.  Calls whose kernels overlap on the GPU
// (for example on two different streams) race on the scratch and give wrong
// results: serialise them.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/wavey_cuda.h"

namespace {

constexpr int NA_CHUNK = 128;
constexpr int NA_MAX_FREQS = WAVEY_NOALLOC_MAX_FREQS;
constexpr int NA_MAX_DEVICES = 64;
constexpr int NA_BLOCK = 256;

static __device__ __align__(256) float2 g_noalloc_twiddles[NA_CHUNK * NA_MAX_FREQS];

// tw[t][f] = exp(-j 2 pi frac(f dt (n0 + t))), the phase formed in FP64 as
// the reference's running DFT forms it (core/wavey-solver/src/fdtd.rs:680).
__global__ void na_twiddles(float2 *tw, const double *freqs, int nf, double dt, long long n0, int count) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count * nf) return;
    const int t = idx / nf, f = idx - t * nf;
    const double x = freqs[f] * dt * (double)(n0 + t);
    const double ph = -6.283185307179586 * (x - trunc(x));
    double s, c;
    sincos(ph, &s, &c);
    tw[idx] = make_float2((float)c, (float)s);
}

// out[r][f] += sum over the chunk of series[r][n0 + t] * tw[t][f].
__global__ void na_accumulate(const float *series, long long steps, const float2 *tw, double *out, long long n_recv,
                              int nf, long long n0, int count) {
    const long long idx = (long long)blockIdx.x * NA_BLOCK + threadIdx.x;
    if (idx >= n_recv * nf) return;
    const long long r = idx / nf;
    const int f = (int)(idx - r * nf);
    const float *src = series + r * steps + n0;
    float re = 0.f, im = 0.f;
    for (int t = 0; t < count; t++) {
        const float v = __ldg(src + t);
        const float2 w = tw[t * nf + f];
        re = fmaf(v, w.x, re);
        im = fmaf(v, w.y, im);
    }
    out[2 * idx] += (double)re;
    out[2 * idx + 1] += (double)im;
}

std::mutex g_mu;
float2 *g_addr[NA_MAX_DEVICES] = {};

void message(char *err, size_t cap, const char *text) {
    if (err && cap) snprintf(err, cap, "%s", text);
}

}  // namespace

extern "C" int wavey_cuda_receiver_dft_noalloc(int device, const float *series, int64_t n_recv, int64_t steps,
                                               const double *freqs, int64_t nf, double dt, double *out, void *stream,
                                               char *err, size_t err_cap) {
    if (device < 0 || device >= NA_MAX_DEVICES) {
        message(err, err_cap, "device index out of range");
        return WAVEY_E_INVALID;
    }
    if (n_recv < 0 || steps < 0 || nf < 0 || !(dt > 0.0)) {
        message(err, err_cap, "negative size or non-positive dt");
        return WAVEY_E_INVALID;
    }
    if (nf > NA_MAX_FREQS) {
        char buf[160];
        snprintf(buf, sizeof buf, "%lld frequencies exceed the fixed scratch of %d frequencies",
                 (long long)nf, NA_MAX_FREQS);
        message(err, err_cap, buf);
        return WAVEY_E_LIMIT;
    }
    if (n_recv * nf == 0) return WAVEY_OK;
    if ((n_recv * nf + NA_BLOCK - 1) / NA_BLOCK >= (1ll << 31)) {
        message(err, err_cap, "too many receivers x frequencies for one launch");
        return WAVEY_E_LIMIT;
    }
    if (!series || !freqs || !out) {
        message(err, err_cap, "null device pointer");
        return WAVEY_E_INVALID;
    }
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        message(err, err_cap, "cannot make the device current");
        return WAVEY_E_CUDA;
    }
    float2 *tw = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_addr[device]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_twiddles);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                cudaSetDevice(prev);
                message(err, err_cap, cudaGetErrorString(e));
                return WAVEY_E_CUDA;
            }
            g_addr[device] = static_cast<float2 *>(p);
        }
        tw = g_addr[device];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(out, 0, (size_t)(n_recv * nf) * 2 * sizeof(double), s);
    for (int64_t n0 = 0; e == cudaSuccess && n0 < steps; n0 += NA_CHUNK) {
        const int count = (int)((steps - n0) < NA_CHUNK ? (steps - n0) : NA_CHUNK);
        const int tw_threads = count * (int)nf;
        na_twiddles<<<(tw_threads + NA_BLOCK - 1) / NA_BLOCK, NA_BLOCK, 0, s>>>(tw, freqs, (int)nf, dt, n0, count);
        const long long total = n_recv * nf;
        na_accumulate<<<(unsigned)((total + NA_BLOCK - 1) / NA_BLOCK), NA_BLOCK, 0, s>>>(series, steps, tw, out, n_recv,
                                                                                         (int)nf, n0, count);
        e = cudaGetLastError();
    }
    cudaSetDevice(prev);
    if (e != cudaSuccess) {
        message(err, err_cap, cudaGetErrorString(e));
        return WAVEY_E_CUDA;
    }
    return WAVEY_OK;
}
