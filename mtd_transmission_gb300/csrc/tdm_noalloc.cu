// Allocation-free off-axis extraction.
//
// Some callers cannot allocate GPU memory: a camera acquisition loop that
// extracts each burst of holograms as it arrives cannot afford cudaMalloc
// (it may synchronise the device and stall the frame loop), and a host
// application whose memory pool already owns the GPU's memory has none to
// give.  tdm_extract_noalloc serves them: it runs the same extraction kernels
// as tdm_extract, on the caller's device buffers and stream, and keeps its
// scratch (the row-pass intermediate) in a fixed array compiled into this
// library.  Every GPU that loads the library holds that array until the
// process exits.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <vector>

#include "extract_kernels.cuh"
#include "host_tables.h"

namespace {

using namespace tdm;
using namespace tdm::extract;

constexpr size_t kScratchBytes = size_t(4) << 20;  // 4 MiB: one 2048 x 256 band, or two 1024 x 256
constexpr int kMaxH = 2048;
constexpr int kWindowLen = 256 + 512 + 1024 + 2048;  // one window table per supported CCD_ROIX

static __device__ __align__(256) float2 g_scratch[kScratchBytes / sizeof(float2)];
static __device__ __align__(256) float2 g_twiddle[kTwTotal];
static __device__ __align__(256) float2 g_window[kWindowLen];

int window_offset(int H) { return H - 256; }  // 256 -> 0, 512 -> 256, 1024 -> 768, 2048 -> 1792

// Device addresses of the arrays above.  In host code the array names are
// host-side stand-ins, not device addresses, so they are looked up once per
// device with cudaGetSymbolAddress while that device is current.
struct Symbols {
    bool ready = false;
    float2* scratch = nullptr;
    float2* twiddle = nullptr;
    float2* window = nullptr;
};
constexpr int kMaxDevices = 64;
std::mutex g_mu;
Symbols g_sym[kMaxDevices];

int device_symbols(int dev, Symbols& out) {
    if (dev < 0 || dev >= kMaxDevices) return TDM_EUNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_mu);
    Symbols& s = g_sym[dev];
    if (!s.ready) {
        if (cudaGetSymbolAddress(reinterpret_cast<void**>(&s.scratch), g_scratch) != cudaSuccess ||
            cudaGetSymbolAddress(reinterpret_cast<void**>(&s.twiddle), g_twiddle) != cudaSuccess ||
            cudaGetSymbolAddress(reinterpret_cast<void**>(&s.window), g_window) != cudaSuccess) {
            cudaGetLastError();
            return TDM_ECUDA;
        }
        const std::vector<float2> tw = twiddle_table();
        std::vector<float2> wt(kWindowLen);
        for (int H = 256; H <= kMaxH; H *= 2) {
            const std::vector<float2> t = hologram_window(H);  // hologram window, main.cpp:105
            std::copy(t.begin(), t.end(), wt.begin() + window_offset(H));
        }
        // A copy from pageable host memory may return before the data has
        // reached the device; the tables must be complete before any kernel
        // on any stream (or another thread that sees ready) reads them.
        if (cudaMemcpy(s.twiddle, tw.data(), kTwTotal * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(s.window, wt.data(), kWindowLen * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaDeviceSynchronize() != cudaSuccess) {
            cudaGetLastError();
            return TDM_ECUDA;
        }
        s.ready = true;
    }
    out = s;
    return TDM_OK;
}

// Device (or managed) memory of device dev.
bool on_device(const void* p, int dev) {
    cudaPointerAttributes at;
    if (!p || cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == dev;
}

template <int H>
int run(const Symbols& s, const void* holos, int bits, int n, float2* out, int F, int x0, int y0,
        cudaStream_t st) {
    using C = ExtractCfg<H>;
    const size_t sm_rows = C::smem_rows(F), sm_cols = C::smem_cols(F);
    if (!window_edge_ok(H, tukey_flat(H, 0.05f), win_edge<H>())) return TDM_EUNSUPPORTED;
    if (sm_rows > 48 * 1024 &&
        cudaFuncSetAttribute(k_extract_rows<H, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_rows))
        return TDM_ECUDA;
    if (sm_cols > 48 * 1024 &&
        cudaFuncSetAttribute(k_extract_cols<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_cols))
        return TDM_ECUDA;
    const size_t per_holo = (size_t)H * F * sizeof(float2);
    const int chunk = (int)(kScratchBytes / per_holo);
    const size_t in_bytes = (size_t)H * H * (bits == 16 ? 2 : 1);
    for (int h0 = 0; h0 < n; h0 += chunk) {
        const int m = n - h0 < chunk ? n - h0 : chunk;
        k_extract_rows<H, false><<<C::grid_rows(m), C::NT, sm_rows, st>>>(
            static_cast<const char*>(holos) + h0 * in_bytes, bits, s.window + window_offset(H), nullptr, s.twiddle,
            s.scratch, F, x0, nullptr, 0u);
        k_extract_cols<H><<<C::grid_cols(F, m), C::NT, sm_cols, st>>>(
            s.scratch, s.twiddle, out + (size_t)h0 * F * F, F, x0, y0, nullptr);
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

}  // namespace

extern "C" int tdm_extract_noalloc(const tdm_geom* geom, const void* holos, int bits, int n, float* spectra_out,
                                   void* stream) {
    if (!geom || !holos || !spectra_out || n <= 0 || (bits != 8 && bits != 16)) return TDM_EINVAL;
    const int H = geom->ccd_roix, N = geom->nxmax, F = 2 * N;
    const int x0 = geom->circle_cx - N, y0 = geom->circle_cy - N;
    if ((H & (H - 1)) || H < 256 || H > kMaxH || (F & (F - 1)) || F < 64 || F > 512) {
        std::fprintf(stderr, "tdm_extract_noalloc: CCD_ROIX must be a power of two in [256, 2048] and 2*NXMAX in [64, 512]\n");
        return TDM_EUNSUPPORTED;
    }
    if (x0 < 0 || y0 < 0 || x0 + F > H || y0 + F > H) {
        std::fprintf(stderr, "tdm_extract_noalloc: crop window outside the hologram spectrum\n");
        return TDM_EINVAL;
    }
    if ((size_t)H * F * sizeof(float2) > kScratchBytes) {
        std::fprintf(stderr,
                     "tdm_extract_noalloc: one %dx%d hologram needs %zu bytes of scratch; the fixed scratch holds %zu "
                     "(CCD_ROIX * 2*NXMAX must not exceed 524288)\n",
                     H, H, (size_t)H * F * sizeof(float2), kScratchBytes);
        return TDM_EUNSUPPORTED;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TDM_ECUDA;
    if (!on_device(holos, dev) || !on_device(spectra_out, dev)) {
        std::fprintf(stderr, "tdm_extract_noalloc: holograms and spectra must be in the current device's memory\n");
        return TDM_EINVAL;
    }
    // the kernels store complex values as float2 and read 16-bit samples as uint16
    if ((reinterpret_cast<uintptr_t>(spectra_out) & 7) || (bits == 16 && (reinterpret_cast<uintptr_t>(holos) & 1))) {
        std::fprintf(stderr, "tdm_extract_noalloc: spectra must be 8-byte aligned and 16-bit holograms 2-byte aligned\n");
        return TDM_EINVAL;
    }
    Symbols s;
    if (int rc = device_symbols(dev, s)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float2* out = reinterpret_cast<float2*>(spectra_out);
    switch (H) {
        case 256: return run<256>(s, holos, bits, n, out, F, x0, y0, st);
        case 512: return run<512>(s, holos, bits, n, out, F, x0, y0, st);
        case 1024: return run<1024>(s, holos, bits, n, out, F, x0, y0, st);
        default: return run<2048>(s, holos, bits, n, out, F, x0, y0, st);
    }
}
