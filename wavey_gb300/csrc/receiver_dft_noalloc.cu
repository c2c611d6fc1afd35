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
// stream capture begins.  The address is remembered together with the
// device's current context; after a device reset (a new primary context, in
// which the library's module is loaded again) the next call looks it up anew.
//
// Every call shares the one scratch array, and each call overwrites it
// completely before reading it, so nothing in it needs clearing; the output
// is cleared by the call itself.  A call queues all of its work while holding
// one process-wide lock, so calls from several host threads on the same
// stream never interleave their kernels.  Calls whose kernels overlap on the
// GPU (for example on two different streams) race on the scratch and give
// wrong results: serialise them.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
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

// Per device: the scratch array's device address and the context it was
// looked up in.
struct ScratchAddr {
    CUcontext ctx;
    float2 *addr;
};
std::mutex g_mu;
ScratchAddr g_addr[NA_MAX_DEVICES] = {};

// The calling thread's current context (cuCtxGetCurrent, fetched from the
// driver once, so that the library needs no link-time libcuda).
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
CUcontext current_context() {
    static CtxGetCurrentFn fn = []() -> CtxGetCurrentFn {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<CtxGetCurrentFn>(p);
        return nullptr;
    }();
    CUcontext c = nullptr;
    if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
    return c;
}

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
    if (nf > 0 && n_recv > INT64_MAX / nf) {
        message(err, err_cap, "too many receivers x frequencies for one launch");
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
    cudaError_t e = cudaSuccess;
    {
        // Held until the last launch is queued: calls from several host
        // threads on one stream then queue their kernels one call after the
        // other, and none reads another's twiddles.
        std::lock_guard<std::mutex> lock(g_mu);
        ScratchAddr &slot = g_addr[device];
        // cudaSetDevice above made the device's primary context current (it
        // initialises it since CUDA 12), so this is the context the kernels
        // run in.
        const CUcontext ctx = current_context();
        if (!slot.addr || !ctx || slot.ctx != ctx) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_twiddles);
            if (e == cudaSuccess && !p) e = cudaErrorInvalidSymbol;
            if (e == cudaSuccess) slot = ScratchAddr{ctx, static_cast<float2 *>(p)};
        }
        float2 *const tw = slot.addr;
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(out, 0, (size_t)(n_recv * nf) * 2 * sizeof(double), s);
        for (int64_t n0 = 0; e == cudaSuccess && n0 < steps; n0 += NA_CHUNK) {
            const int count = (int)((steps - n0) < NA_CHUNK ? (steps - n0) : NA_CHUNK);
            const int tw_threads = count * (int)nf;
            na_twiddles<<<(tw_threads + NA_BLOCK - 1) / NA_BLOCK, NA_BLOCK, 0, s>>>(tw, freqs, (int)nf, dt, n0, count);
            const long long total = n_recv * nf;
            na_accumulate<<<(unsigned)((total + NA_BLOCK - 1) / NA_BLOCK), NA_BLOCK, 0, s>>>(series, steps, tw, out,
                                                                                             n_recv, (int)nf, n0, count);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) cudaGetLastError();
    cudaSetDevice(prev);
    if (e != cudaSuccess) {
        message(err, err_cap, cudaGetErrorString(e));
        return WAVEY_E_CUDA;
    }
    return WAVEY_OK;
}
