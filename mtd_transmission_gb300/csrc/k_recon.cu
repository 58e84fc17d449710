// Reconstruction (Reconstruction/main.cpp:203-352).
//
// Per field (main.cpp:207-217): x Tukey(0.1), shift by (N, N), forward FFT x dx^2,
// shift by posSpec.  With k the FFT bin, the value that retroPropag_Born reads
// at cap pixel fd = ((k + posSpec) mod F) - N is
//     (-1)^(kx+ky) dx^2 FFT2(field * tukey)[k],
// so the per-field kernels work on natural FFT bins and store, per bin, the
// cap contribution -2i k0 sdz value (cteUb2Pot*cteNorm*sdz, fonctions.cpp:902,927),
// 0 outside the cap cells (an 8-byte cap value), and the cell's volume plane z
// (-1 outside the NA disc) as a 2-byte integer: the gather reads the planes of
// the bins that fall in its column and the values of the cells that hit it.
//
// Mapping (retroPropag_Born, src/fonctions.cpp:875-935) as a gather: voxel
// column (X, Y) reads bin kx = (X - D/2) mod F for every angle whose cap window
// covers it; each angle hits a column at most once, so the column's sums are
// formed without atomics, in a fixed order; hit counts are exact (k_gather_z).
//
// Volume: fftshift3D, backward 3D FFT x Delta_f^3, fftshift3D, x -1/(2 n0 kv^2)
// (main.cpp:282-352).  For even D the two shifts are sign modulations:
//     out[m] = (-1)^(mx+my+mz+3D/2) IFFT3((-1)^(kx+ky+kz) V)[m].
// The z pass runs inside the gather (k_gather_z); then a y pass, and an x pass
// that writes the index and absorption volumes.
#include "tdm_internal.cuh"
#include "fft_warp.cuh"
#include "form.cuh"
#include "fp_bits.cuh"
#include "cap_geometry.cuh"

namespace tdm {
namespace {

template <class K>
cudaError_t allow_smem(K kernel, size_t bytes) {
    return max_dynamic_smem(reinterpret_cast<const void*>(kernel), bytes);
}

template <int F>
struct CapCfg {
    using W = WarpFFT<F>;
    static constexpr int B = 8 * W::G;    // transforms per CTA
    static constexpr int NT = B * W::T;   // 256 threads
    static constexpr size_t SMEM = (size_t)B * W::STRIDE * sizeof(float2);
};

template <int F>
__global__ void __launch_bounds__(CapCfg<F>::NT)
k_cap_rows(const float2* __restrict__ fields, const float* __restrict__ tuk, int2 flat, const float2* __restrict__ tw,
           float2* __restrict__ r1) {
    using C = CapCfg<F>;
    using W = typename C::W;
    constexpr int T = W::T, E = W::E;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / T, j = threadIdx.x % T;
    const int a = blockIdx.y, y = blockIdx.x * C::B + tr;
    const float wy = tuk[y];
    const float2* src = fields + ((size_t)a * F + y) * F;
    float2 x[E];
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) {
        const int xx = j + n1 * T;
        x[n1] = c_scale(src[xx], ((xx >= flat.x && xx <= flat.y) ? 1.0f : __ldg(&tuk[xx])) * wy);
    }
    fft_warp_regs<F, -1>(x, sm + tr * W::STRIDE, j, tw);
    float2* dst = r1 + ((size_t)a * F + y) * F;
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) dst[j + q * T + E * k2] = x[q * T + k2];
    }
}

// k_cap_rows with the field formed on the fly from the chunk's unwrapped
// phase, amplitude and fits (the field stage's k_form, same arithmetic); the
// field is also stored, as k_form would.
template <int F>
__global__ void __launch_bounds__(CapCfg<F>::NT)
k_cap_rows_form(const float* __restrict__ unwrapped, const float* __restrict__ amp, const double* __restrict__ beta,
                int born, const float* __restrict__ tuk, int2 flat, const float2* __restrict__ tw,
                float2* __restrict__ fields,
                float2* __restrict__ r1) {
    using C = CapCfg<F>;
    using W = typename C::W;
    constexpr int T = W::T, E = W::E;
    extern __shared__ float2 sm[];
    __shared__ float bf[2 * kNC];
    if (threadIdx.x < 2 * kNC) bf[threadIdx.x] = (float)beta[(size_t)blockIdx.y * 2 * kNC + threadIdx.x];
    __syncthreads();
    const int tr = threadIdx.x / T, j = threadIdx.x % T;
    const int a = blockIdx.y, y = blockIdx.x * C::B + tr;
    const float wy = tuk[y];
    const size_t row = ((size_t)a * F + y) * F;
    const FormRow fr = form_row(bf, y, F);
    float2 x[E];
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) {
        const int xx = j + n1 * T;
        const float2 f = form_value(fr, xx, F, unwrapped[row + xx], amp[row + xx], born);
        fields[row + xx] = f;
        x[n1] = c_scale(f, ((xx >= flat.x && xx <= flat.y) ? 1.0f : __ldg(&tuk[xx])) * wy);
    }
    fft_warp_regs<F, -1>(x, sm + tr * W::STRIDE, j, tw);
    float2* dst = r1 + row;
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) dst[j + q * T + E * k2] = x[q * T + k2];
    }
}

template <int F>
__global__ void __launch_bounds__(CapCfg<F>::NT)
k_cap_cols(const float2* __restrict__ r1, const int2* __restrict__ posspec, const double* __restrict__ s_tab,
           const float* __restrict__ s_tabf, Params p, const float2* __restrict__ tw, float2* __restrict__ rec,
           int16_t* __restrict__ recz, int* __restrict__ err) {
    using C = CapCfg<F>;
    using W = typename C::W;
    constexpr int B = C::B, NT = C::NT;
    extern __shared__ float2 sm[];
    __shared__ double s_fz;
    const int tr = threadIdx.x / W::T, j = threadIdx.x % W::T;
    const int a = blockIdx.y, kx0 = blockIdx.x * B;
    const int2 ps = posspec[a];
    if (threadIdx.x == 0) s_fz = cap_fzm0(p, ps);
#pragma unroll  // every load in flight before the first store
    for (int r = 0; r < B * F / NT; ++r) {
        const int i = threadIdx.x + r * NT, t = i % B, ky = i / B;
        sm[t * W::STRIDE + W::pad(ky)] = r1[((size_t)a * F + ky) * F + kx0 + t];
    }
    __syncthreads();
    fft_warp<F, -1>(sm + tr * W::STRIDE, j, tw);
    __syncthreads();
    const double fz = s_fz;
    const float fzf = (float)fz, ir = (float)p.inv_rayon;
#pragma unroll 2
    for (int r = 0; r < B * F / NT; ++r) {
        const int i = threadIdx.x + r * NT, t = i % B, ky = i / B, kx = kx0 + t;
        const size_t o = ((size_t)a * F + ky) * F + kx;
        float sf = 0.f;
        const int z = cap_plane(p, ps, fz, fzf, kx, ky, s_tab, s_tabf, &sf, err);
        float2 val = make_float2(0.f, 0.f);
        if (z >= 0) {
            const float2 v = sm[t * W::STRIDE + W::pad(ky)];
            const float Bc = cap_weight(p, sf, ir, kx, ky);
            val = make_float2(-Bc * v.y, Bc * v.x);
        }
        rec[o] = val;
        recz[o] = (int16_t)z;
    }
}

// ---------------------------------------------------------------- cap accumulation
// One warp per voxel column (X, Y); a CTA covers 32 consecutive X at one Y.
// An angle's cap window is the F x F bins around its specular position, so a
// column is covered by a fraction of the angles: the CTA first lists, in
// ascending order, the angles whose window covers row Y and any of its 32
// columns.  The lanes then take 32 consecutive listed angles at a time: each
// lane loads its angle's cell plane in the column (a 2-byte record), and the
// cap value only when the bin is a cap cell; the planes of the next two groups
// and the values of the next group are loaded while the current one is
// added, and groups without a hit are skipped.  An angle hits a column at
// most once, at one plane, and
// the column's running sums live in FP64 in shared memory.  When the group's
// planes are distinct (seen through a plane -> lane ownership table) every
// lane adds its own hit; otherwise lanes sharing a plane are grouped and the
// group's lowest lane sums the members in ascending angle order (FP32, at
// most 32 terms) before adding the sum.  The sums are deterministic, the hit
// counts exact.  Widening the FP32 hits and narrowing the sums are done on
// the integer pipe (fp_bits.cuh), so the FP64 pipe only adds.

// Lists, in ascending order, the angles whose window covers row Y (by = Y -
// D/2) and one of the columns bx0 .. bx0 + 31 of the CTA: list[i] = (posSpec
// x, angle).  Returns the count; all NW warps of the CTA call it together.
template <int NW>
__device__ __forceinline__ int list_angles(const int2* __restrict__ posspec, int M, int F, int by, int bx0, int2* list,
                                           int* s_wc, int* s_listed) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) *s_listed = 0;
    __syncthreads();
    for (int a0 = 0; a0 < M; a0 += NW * 32) {
        const int a = a0 + threadIdx.x;
        int2 q = make_int2(0, 0);
        bool keep = false;
        if (a < M) {
            q = posspec[a];
            keep = (unsigned)(by + q.y) < (unsigned)F && bx0 + 31 + q.x >= 0 && bx0 + q.x < F;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) s_wc[w] = __popc(bal);
        __syncthreads();
        int off = *s_listed;
        for (int k = 0; k < w; ++k) off += s_wc[k];
        if (keep) list[off + __popc(bal & ((1u << lane) - 1u))] = make_int2(q.x, a);
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = *s_listed;
            for (int k = 0; k < NW; ++k) t += s_wc[k];
            *s_listed = t;
        }
        __syncthreads();
    }
    return *s_listed;
}

// One warp sums column (bx, by) of the listed angles into acc / cnt (band
// entries, zeroed here): the cells' planes and values are read from the cap
// records at koff, the bin of the column in each angle's F x F window.
__device__ __forceinline__ void gather_column(const float2* __restrict__ rec, const int16_t* __restrict__ recz,
                                              const int2* list, int listed, size_t FF, size_t koff, int bx, int F,
                                              int zmin, int band, double2* acc, uint16_t* cnt, uint8_t* own,
                                              float2* stg, int lane) {
    for (int e = lane; e < band; e += 32) {
        acc[e] = make_double2(0.0, 0.0);
        cnt[e] = 0;
    }
    // plane of listed angle i's cell in this column, or -1 when the angle's
    // window misses the column or the bin is outside its cap; the cap
    // value of a cell with plane z
    auto fetch_z = [&](int i) {
        int z = -1;
        if (i < listed) {
            const int2 q = list[i];
            if ((unsigned)(bx + q.x) < (unsigned)F) z = __ldg(&recz[(size_t)q.y * FF + koff]);
        }
        return z;
    };
    auto fetch_v = [&](int i, int z) {
        return z >= 0 ? __ldg(&rec[(size_t)list[i].y * FF + koff]) : make_float2(0.f, 0.f);
    };
    int z_nxt = fetch_z(lane), z_nxt2 = fetch_z(32 + lane);
    float2 v_nxt = fetch_v(lane, z_nxt);
    __syncwarp();
    for (int g0 = 0; g0 < listed; g0 += 32) {
        const int z = z_nxt;
        const float2 r = v_nxt;
        z_nxt = z_nxt2;
        v_nxt = fetch_v(g0 + 32 + lane, z_nxt);
        z_nxt2 = fetch_z(g0 + 64 + lane);
        const int e = z >= 0 ? z - zmin : -1;
        if (!__any_sync(0xffffffffu, e >= 0)) continue;
        if (e >= 0) own[e] = (uint8_t)lane;
        __syncwarp();
        const bool shared_plane = e >= 0 && own[e] != lane;
        if (!__any_sync(0xffffffffu, shared_plane)) {
            if (e >= 0) {
                double2 t = acc[e];
                t.x += widen(r.x);
                t.y += widen(r.y);
                acc[e] = t;
                cnt[e]++;
            }
        } else {
            const unsigned grp = __match_any_sync(0xffffffffu, e >= 0 ? e : -1 - lane);
            stg[lane] = make_float2(r.x, r.y);
            __syncwarp();
            if (e >= 0 && (grp & ((1u << lane) - 1)) == 0) {  // lowest lane of its plane group
                float sx = 0.0f, sy = 0.0f;
                for (unsigned g = grp; g; g &= g - 1) {
                    const float2 u = stg[__ffs(g) - 1];
                    sx += u.x;
                    sy += u.y;
                }
                double2 t = acc[e];
                t.x += widen(sx);
                t.y += widen(sy);
                acc[e] = t;
                cnt[e] += (uint16_t)__popc(grp);
            }
        }
        __syncwarp();
    }
}

// Cell (X, Y, zmin + e) of the normalised spectrum from its sums (main.cpp:243-249;
// not normalised for the adjoint scatter); (-1)^(X+Y+Z) stands for the first
// fftshift3D.
__device__ __forceinline__ float2 gather_cell(const double2* acc, const uint16_t* cnt, int e, int X, int Y, int zmin,
                                              int normalize, unsigned& n) {
    n = cnt[e];
    float2 val = make_float2(0.0f, 0.0f);
    if (n) {
        const double2 t = acc[e];
        const float dn = normalize ? (float)n : 1.0f;  // FP32 division: FP64 division is a long sequence here
        val = make_float2(narrow(t.x) / dn, narrow(t.y) / dn);
    }
    if ((X + Y + zmin + e) & 1) val = make_float2(-val.x, -val.y);
    return val;
}

// ---------------------------------------------------------------- gather fused with the z pass
// k_gather_z: the cap gather and the inverse FFT along z (the first axis of
// the 3D inverse FFT) in one kernel, so that the cap band (the planes of the
// spectrum that caps reach) is neither written to HBM nor read back.  A CTA
// of kGZ warps covers 32 consecutive columns (X) at one Y; a warp takes its
// columns G = WarpFFT<D>::G at a time (the lanes of one column transform),
// sums each with gather_column into its own FP64 sums, loads the G
// normalised columns into registers (zero outside the band) and
// inverse-transforms them along z together.  The transform's exchange
// buffers (T (T + 1) slots per transform, fft_warp_regs_lean) overlay the
// sums, which are in registers by then.  Each lane stores its outputs
// directly (lane-minor order is contiguous in z) into the [y][x][z] volume.
// The OTF mask (Re != 0 after normalisation, main.cpp:262-267) of the CTA's
// 32 columns is collected as one bit per column and plane in shared memory
// and stored as 32-byte rows; planes outside the band are cleared by the
// host.
constexpr int kGZ = 4;  // warps per CTA

template <int D>
struct GatherZ {
    using W = WarpFFT<D>;
    static constexpr int G = W::G, T = W::T, E = W::E;
    static constexpr int COLS = 32 / kGZ;  // columns per warp
    static_assert(COLS % G == 0, "a warp's columns split into groups of G");
    // per-warp region: G sums (double2) and G counts (uint16) of the band, or,
    // once the sums are in registers, the G exchange buffers
    __host__ __device__ static size_t region(int band) {
        const size_t sums = (size_t)G * band * (sizeof(double2) + sizeof(uint16_t));
        const size_t xch = (size_t)G * T * (T + 1) * sizeof(float2);
        return ((sums > xch ? sums : xch) + 15) & ~size_t(15);
    }
    __host__ __device__ static size_t own_bytes(int band) { return (size_t)((band + 15) & ~15); }
    static size_t smem(int band, int n) {
        return kGZ * (region(band) + 32 * sizeof(float2) + own_bytes(band)) + (((size_t)band * 4 + 7) & ~size_t(7)) +
               (size_t)n * sizeof(int2);
    }
};

template <int D>
__global__ void __launch_bounds__(kGZ * 32, 5)
k_gather_z(const float2* __restrict__ rec, const int16_t* __restrict__ recz, const int2* __restrict__ posspec, int M,
           Params p, const float2* __restrict__ tw, float2* __restrict__ vol, uint32_t* __restrict__ cnt_out,
           uint8_t* __restrict__ otf, int normalize) {
    using Z = GatherZ<D>;
    constexpr int G = Z::G, T = Z::T, E = Z::E;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ int s_wc[kGZ];
    __shared__ int s_listed;
    const int band = p.band;
    const size_t reg = Z::region(band), ownb = Z::own_bytes(band);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* region = smraw + w * reg;
    double2* acc0 = reinterpret_cast<double2*>(region);                  // G x band
    uint16_t* cnt0 = reinterpret_cast<uint16_t*>(acc0 + G * band);      // G x band
    float2* stg = reinterpret_cast<float2*>(smraw + kGZ * reg) + w * 32;
    uint8_t* own = smraw + kGZ * (reg + 32 * sizeof(float2)) + w * ownb;
    uint32_t* bits = reinterpret_cast<uint32_t*>(smraw + kGZ * (reg + 32 * sizeof(float2) + ownb));  // band
    int2* list = reinterpret_cast<int2*>(reinterpret_cast<unsigned char*>(bits) + (((size_t)band * 4 + 7) & ~size_t(7)));
    const int F = p.F, h = D / 2, zmin = p.zmin;
    const size_t FF = (size_t)F * F;
    const int Y = blockIdx.y, by = Y - h, X0 = blockIdx.x * 32;
    if (otf)
        for (int e = threadIdx.x; e < band; e += kGZ * 32) bits[e] = 0;  // ordered by list_angles' barriers
    const int listed = list_angles<kGZ>(posspec, M, F, by, X0 - h, list, s_wc, &s_listed);
    const int g = lane / T, j = lane % T;  // this lane's transform of the group, and its lane in it
    for (int r = 0; r < Z::COLS / G; ++r) {
#pragma unroll 1
        for (int gg = 0; gg < G; ++gg) {
            const int X = X0 + w + kGZ * (r * G + gg);
            const int bx = X - h;
            const size_t koff = (size_t)(((by % F) + F) % F) * F + ((bx % F) + F) % F;
            double2* acc = acc0 + gg * band;
            const uint16_t* cnt = cnt0 + gg * band;
            gather_column(rec, recz, list, listed, FF, koff, bx, F, zmin, band, acc, cnt0 + gg * band, own, stg,
                          lane);
            // normalised cells, in place: cell e's float2 goes to bytes [8e, 8e + 8), over sums of cells
            // below the current 32, which have been read (a rolled loop keeps the kernel's code small)
            float2* cell = reinterpret_cast<float2*>(acc);
            for (int e0 = 0; e0 < band; e0 += 32) {
                const int e = e0 + lane;
                float2 v = make_float2(0.f, 0.f);
                if (e < band) {
                    unsigned n;
                    v = gather_cell(acc, cnt, e, X, Y, zmin, normalize, n);
                    if (cnt_out) cnt_out[((size_t)(zmin + e) * D + Y) * D + X] = n;
                    if (otf && v.x != 0.0f) atomicOr(&bits[e], 1u << (X - X0));
                }
                __syncwarp();
                if (e < band) cell[e] = v;
            }
        }
        __syncwarp();
        const int X = X0 + w + kGZ * (r * G + g);
        const float2* cell = reinterpret_cast<const float2*>(acc0 + g * band);
        float2 x[E];
#pragma unroll
        for (int n1 = 0; n1 < E; ++n1) {
            const int e = j + n1 * T - zmin;
            x[n1] = (unsigned)e < (unsigned)band ? cell[e] : make_float2(0.f, 0.f);
        }
        // the exchange buffers overlay the sums: every lane has read its column (the transform's first __syncwarp)
        fft_warp_regs_lean<D, +1>(x, reinterpret_cast<float2*>(region) + g * T * (T + 1), j, tw);
        float2* col = vol + ((size_t)Y * D + X) * D;
#pragma unroll
        for (int q = 0; q < E / T; ++q) {
#pragma unroll
            for (int k2 = 0; k2 < T; ++k2) col[j + q * T + E * k2] = x[q * T + k2];
        }
        __syncwarp();  // the next group's sums overlay the exchange buffers
    }
    if (otf) {
        __syncthreads();
        uint8_t* o = otf + (size_t)Y * D + X0;
        const size_t plane = (size_t)D * D;
        if ((reinterpret_cast<uintptr_t>(otf) & 15) == 0) {
            for (int i = threadIdx.x; i < 2 * band; i += kGZ * 32) {  // 16 columns' flags per store
                const uint32_t b = bits[i >> 1] >> (16 * (i & 1));
                uint32_t v[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const uint32_t nib = (b >> (4 * t)) & 0xFu;
                    v[t] = (nib & 1u) | ((nib & 2u) << 7) | ((nib & 4u) << 14) | ((nib & 8u) << 21);
                }
                *reinterpret_cast<uint4*>(o + (size_t)(zmin + (i >> 1)) * plane + 16 * (i & 1)) =
                    make_uint4(v[0], v[1], v[2], v[3]);
            }
        } else {
            for (int i = threadIdx.x; i < 32 * band; i += kGZ * 32)
                o[(size_t)(zmin + i / 32) * plane + i % 32] = (uint8_t)((bits[i / 32] >> (i % 32)) & 1u);
        }
    }
}

template <int D>
struct PassCfg {
    using W = WarpFFT<D>;
    static constexpr int B = 16;           // transforms per CTA
    static constexpr int NT = B * W::T;    // threads per CTA
    static constexpr size_t SMEM = (size_t)B * W::STRIDE * sizeof(float2);
};

// Inverse FFT along y, in place, for B consecutive z at fixed x.
template <int D, int DIR>
__global__ void __launch_bounds__(PassCfg<D>::NT)
k_ypass(float2* __restrict__ vol, const float2* __restrict__ tw) {
    using C = PassCfg<D>;
    using W = typename C::W;
    constexpr int B = C::B, NT = C::NT;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / W::T, j = threadIdx.x % W::T;
    const int z0 = blockIdx.x * B, X = blockIdx.y;
#pragma unroll  // every load in flight before the first store (latency-bound at 8)
    for (int r = 0; r < B * D / NT; ++r) {
        const int i = threadIdx.x + r * NT, t = i % B, Y = i / B;
        sm[t * W::STRIDE + W::pad(Y)] = vol[((size_t)Y * D + X) * D + z0 + t];
    }
    __syncthreads();
    fft_warp<D, DIR>(sm + tr * W::STRIDE, j, tw);
    __syncthreads();
#pragma unroll 8
    for (int r = 0; r < B * D / NT; ++r) {
        const int i = threadIdx.x + r * NT, t = i % B, Y = i / B;
        vol[((size_t)Y * D + X) * D + z0 + t] = sm[t * W::STRIDE + W::pad(Y)];
    }
}

// Inverse FFT along x for B consecutive z at fixed y, scaled and sign-modulated,
// written as the index (real) and absorption (imaginary) volumes, x fastest.
template <int D>
__global__ void __launch_bounds__(PassCfg<D>::NT)
k_xpass(const float2* __restrict__ vol, const float2* __restrict__ tw, float scale, int zblock0, float* __restrict__ re,
        float* __restrict__ im) {
    using C = PassCfg<D>;
    using W = typename C::W;
    constexpr int B = C::B, NT = C::NT;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / W::T, j = threadIdx.x % W::T;
    const int z0 = (zblock0 + blockIdx.x) * B, Y = blockIdx.y;
#pragma unroll  // every load in flight before the first store (latency-bound at 8)
    for (int r = 0; r < B * D / NT; ++r) {
        const int i = threadIdx.x + r * NT, t = i % B, X = i / B;
        sm[t * W::STRIDE + W::pad(X)] = vol[((size_t)Y * D + X) * D + z0 + t];
    }
    __syncthreads();
    fft_warp<D, +1>(sm + tr * W::STRIDE, j, tw);
    __syncthreads();
    const int par = (3 * (D / 2)) & 1;
#pragma unroll 8
    for (int r = 0; r < B * D / NT; ++r) {
        const int i = threadIdx.x + r * NT, t = i / D, X = i % D, Z = z0 + t;
        const float2 v = sm[t * W::STRIDE + W::pad(X)];
        const float sg = ((X + Y + Z + par) & 1) ? -scale : scale;
        const size_t o = ((size_t)Z * D + Y) * D + X;
        if (re) re[o] = v.x * sg;
        if (im) im[o] = v.y * sg;
    }
}

// ---------------------------------------------------------------- forward operator and adjoint
// With the unknown volume x = index + i absorption ([z][y][x], x fastest) and
// s = out_scale, the volume stage above is x = T(V) = s M_out IFFT3(M_in V)
// (unnormalised IFFT, M the fftshift sign patterns).  The forward operator
// is A = S G with G = T^-1 = M_in FFT3(M_out x) / (s D^3) and S the sampling
// of each angle's cap cells (the cells the gather fills, same geometry); its
// adjoint is A^H = G^H S^H, G^H = M_out IFFT3(M_in .) / (s D^3) and S^H the
// unnormalised scatter, i.e. k_gather_z without the division by the hit
// count, followed by the y and x passes with scale 1 / (s D^3).

// Forward x pass: FFT along x of B consecutive z rows at fixed y of the
// index/absorption volumes (x M_out x scale), into the [y][x][z] spectrum.
template <int D>
__global__ void __launch_bounds__(PassCfg<D>::NT)
k_fxpass(const float* __restrict__ re, const float* __restrict__ im, const float2* __restrict__ tw, float scale,
         float2* __restrict__ vol) {
    using C = PassCfg<D>;
    using W = typename C::W;
    constexpr int B = C::B, NT = C::NT;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / W::T, j = threadIdx.x % W::T;
    const int z0 = blockIdx.x * B, Y = blockIdx.y;
    const int par = (3 * (D / 2)) & 1;
#pragma unroll  // every load in flight before the first store
    for (int r = 0; r < B * D / NT; ++r) {
        const int i = threadIdx.x + r * NT, t = i / D, X = i % D, Z = z0 + t;
        const size_t o = ((size_t)Z * D + Y) * D + X;
        const float sg = ((X + Y + Z + par) & 1) ? -scale : scale;
        sm[t * W::STRIDE + W::pad(X)] = make_float2(re[o] * sg, im ? im[o] * sg : 0.0f);
    }
    __syncthreads();
    fft_warp<D, -1>(sm + tr * W::STRIDE, j, tw);
    __syncthreads();
#pragma unroll 8
    for (int r = 0; r < B * D / NT; ++r) {
        const int i = threadIdx.x + r * NT, t = i % B, X = i / B;
        vol[((size_t)Y * D + X) * D + z0 + t] = sm[t * W::STRIDE + W::pad(X)];
    }
}

// Forward z pass: FFT along z of B columns (all planes in), x M_in, only the
// cap band written (the sampling reads nothing else).
template <int D>
__global__ void __launch_bounds__(PassCfg<D>::NT)
k_fzpass(float2* __restrict__ vol, const float2* __restrict__ tw, int zmin, int band) {
    using C = PassCfg<D>;
    using W = typename C::W;
    constexpr int B = C::B, T = W::T, E = W::E;
    extern __shared__ float2 sm[];
    const int t = threadIdx.x / T, j = threadIdx.x % T;
    const size_t c = (size_t)blockIdx.x * B + t;  // y * D + x
    const int XY = (int)(c % D) + (int)(c / D);
    float2* col = vol + c * D;
    float2 x[E];
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) x[n1] = col[j + n1 * T];
    fft_warp_regs<D, -1>(x, sm + t * W::STRIDE, j, tw);
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) {
            const int Z = j + q * T + E * k2;
            if (Z >= zmin && Z < zmin + band) {
                const float2 v = x[q * T + k2];
                col[Z] = ((XY + Z) & 1) ? make_float2(-v.x, -v.y) : v;
            }
        }
    }
}

// Cap values of the spectrum: for each angle and FFT bin, the spectrum at its
// cap cell (0 outside the cap).  With data (cap values of measurements), the
// residual spectrum - data on the cap cells (0 elsewhere) and the misfit
// sum |residual|^2 added to *misfit.
__global__ void __launch_bounds__(256)
k_cap_sample(const float2* __restrict__ vol, const int2* __restrict__ posspec, Params p,
             const double* __restrict__ s_tab, const float* __restrict__ s_tabf, const float2* __restrict__ data,
             float2* __restrict__ caps, float2* __restrict__ res, int16_t* __restrict__ resz, double* __restrict__ misfit,
             int* __restrict__ err) {
    const int a = blockIdx.y, F = p.F, D = p.D;
    const int2 ps = posspec[a];
    __shared__ double s_fz;
    __shared__ double red[8];
    if (threadIdx.x == 0) s_fz = cap_fzm0(p, ps);
    __syncthreads();
    const double fz = s_fz;
    const float fzf = (float)fz;
    double m2 = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < F * F; i += gridDim.x * blockDim.x) {
        const int kx = i % F, ky = i / F;
        const size_t o = (size_t)a * F * F + i;
        float sf;
        const int z = cap_plane(p, ps, fz, fzf, kx, ky, s_tab, s_tabf, &sf, err);
        float2 v = make_float2(0.f, 0.f);
        if (z >= 0) {
            const float2 d = data ? data[o] : make_float2(0.f, 0.f);
            const int X = cap_col(p, kx, ps.x), Y = cap_col(p, ky, ps.y);
            v = vol[((size_t)Y * D + X) * D + z];
            v = make_float2(v.x - d.x, v.y - d.y);
            m2 += (double)v.x * v.x + (double)v.y * v.y;
        }
        if (caps) caps[o] = v;
        if (res) {
            res[o] = v;
            resz[o] = (int16_t)z;
        }
    }
    if (misfit) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) m2 += __shfl_down_sync(0xffffffffu, m2, off);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m2;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
            atomicAdd(misfit, t);
        }
    }
}

// Cap values of given values on the cap cells (0 elsewhere), for the scatter.
__global__ void __launch_bounds__(256)
k_cap_pack(const float2* __restrict__ caps, const int2* __restrict__ posspec, Params p,
           const double* __restrict__ s_tab, const float* __restrict__ s_tabf, float2* __restrict__ rec,
           int16_t* __restrict__ recz, int* __restrict__ err) {
    const int a = blockIdx.y, F = p.F;
    const int2 ps = posspec[a];
    __shared__ double s_fz;
    if (threadIdx.x == 0) s_fz = cap_fzm0(p, ps);
    __syncthreads();
    const double fz = s_fz;
    const float fzf = (float)fz;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < F * F; i += gridDim.x * blockDim.x) {
        const size_t o = (size_t)a * F * F + i;
        float sf;
        const int z = cap_plane(p, ps, fz, fzf, i % F, i / F, s_tab, s_tabf, &sf, err);
        const float2 v = z >= 0 ? caps[o] : make_float2(0.f, 0.f);
        rec[o] = v;
        recz[o] = (int16_t)z;
    }
}

// One projected-gradient step of the regularised reconstruction, per voxel of
// the [z][y][x] volumes: x <- clamp(x - step g - tv dTV(x)) (tv per channel),
// for the index (real part) and, when present, the absorption.  TV is the
// isotropic total variation with forward differences (zero across the far
// faces) smoothed by eps: sum sqrt(|grad x|^2 + eps^2).
__device__ __forceinline__ float tv_grad(const float* __restrict__ x, int D, int X, int Y, int Z, float eps2) {
    const size_t sy = D, sz = (size_t)D * D;
    auto at = [&](int x_, int y_, int z_) { return x[(size_t)z_ * sz + (size_t)y_ * sy + x_]; };
    // gradient of the cell anchored at (x_, y_, z_) and its norm
    auto cell = [&](int x_, int y_, int z_, float& gx, float& gy, float& gz) {
        const float c = at(x_, y_, z_);
        gx = x_ + 1 < D ? at(x_ + 1, y_, z_) - c : 0.0f;
        gy = y_ + 1 < D ? at(x_, y_ + 1, z_) - c : 0.0f;
        gz = z_ + 1 < D ? at(x_, y_, z_ + 1) - c : 0.0f;
        return rsqrtf(gx * gx + gy * gy + gz * gz + eps2);
    };
    float gx, gy, gz;
    float inv = cell(X, Y, Z, gx, gy, gz);
    float g = -(gx + gy + gz) * inv;
    if (X > 0) { inv = cell(X - 1, Y, Z, gx, gy, gz); g += gx * inv; }
    if (Y > 0) { inv = cell(X, Y - 1, Z, gx, gy, gz); g += gy * inv; }
    if (Z > 0) { inv = cell(X, Y, Z - 1, gx, gy, gz); g += gz * inv; }
    return g;
}

__global__ void __launch_bounds__(256)
k_tv_step(const float* __restrict__ xn, const float* __restrict__ xk, const float* __restrict__ gn,
          const float* __restrict__ gk, int D, float step, float tv_n, float tv_k, float eps2, float nlo, float nhi,
          float klo, float khi, float* __restrict__ xn_out, float* __restrict__ xk_out) {
    const size_t total = (size_t)D * D * D;
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < total; v += (size_t)gridDim.x * blockDim.x) {
        const int X = (int)(v % D), Y = (int)((v / D) % D), Z = (int)(v / ((size_t)D * D));
        float a = xn[v] - step * gn[v];
        if (tv_n != 0.0f) a -= tv_n * tv_grad(xn, D, X, Y, Z, eps2);
        xn_out[v] = fminf(fmaxf(a, nlo), nhi);
        if (xk) {
            float b = xk[v] - step * gk[v];
            if (tv_k != 0.0f) b -= tv_k * tv_grad(xk, D, X, Y, Z, eps2);
            xk_out[v] = fminf(fmaxf(b, klo), khi);
        }
    }
}

template <int F>
int cap_impl(tdm_ctx* c, int a0, int n, bool form) {
    using C = CapCfg<F>;
    Buffers& b = c->b;
    if (allow_smem(k_cap_rows<F>, C::SMEM) || allow_smem(k_cap_rows_form<F>, C::SMEM) ||
        allow_smem(k_cap_cols<F>, C::SMEM))
        return TDM_ECUDA;
    if (form && n > c->chunk) return TDM_EINVAL;  // the chunk buffers hold one chunk
    const size_t FF = (size_t)F * F;
    for (int g0 = a0; g0 < a0 + n; g0 += c->chunk) {
        const int m = a0 + n - g0 < c->chunk ? a0 + n - g0 : c->chunk;
        if (form) {
            Launch l(c, K_CAP_ROWS);
            k_cap_rows_form<F><<<dim3(F / C::B, m), C::NT, C::SMEM, c->stream>>>(
                c->p.deroul ? b.unwrapped : b.phase, b.amp, b.beta, c->p.born, b.tuk_f, c->tuk_f_flat, b.tw,
                b.fields + g0 * FF, b.r1);
        } else {
            Launch l(c, K_CAP_ROWS);
            k_cap_rows<F><<<dim3(F / C::B, m), C::NT, C::SMEM, c->stream>>>(b.fields + g0 * FF, b.tuk_f,
                                                                             c->tuk_f_flat, b.tw, b.r1);
        }
        {
            Launch l(c, K_CAP_COLS);
            k_cap_cols<F><<<dim3(F / C::B, m), C::NT, C::SMEM, c->stream>>>(
                b.r1, b.posspec + g0, b.s_tab, b.s_tabf, c->p, b.tw, b.rec.val + g0 * FF, b.rec.z + g0 * FF, b.err);
        }
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

// Download of bytes from a device buffer to host memory on the download
// stream, after the work queued so far on st.
static cudaError_t download_after(tdm_ctx* c, cudaStream_t st, cudaEvent_t ev, void* host, const void* dev,
                                  size_t bytes) {
    cudaError_t e = cudaEventRecord(ev, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->dl_stream, ev, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->dl_stream);
    return e;
}

template <int D>
int volume_impl(tdm_ctx* c, int n, const VolumeOut& out, cudaStream_t st, CapRecs rec, const int2* posspec,
                cudaEvent_t ev_gathered) {
    float* re = out.re;
    float* im = out.im;
    uint8_t* otf = out.otf;
    uint32_t* cnt = out.cnt;
    using P = PassCfg<D>;
    Buffers& b = c->b;
    const Params& p = c->p;
    const size_t sm_a = GatherZ<D>::smem(p.band, n);
    const size_t sm_p = P::SMEM;
    if (sm_a > kMaxSmemPerCta) return TDM_EUNSUPPORTED;
    if (allow_smem(k_gather_z<D>, sm_a) || allow_smem(k_ypass<D, 1>, sm_p) || allow_smem(k_xpass<D>, sm_p))
        return TDM_ECUDA;
    // A staged output part may still be downloading from the previous volume:
    // each part's writer waits for that part's download (ev_dl) just before it runs.
    auto staged_free = [&](int part) { return cudaStreamWaitEvent(st, c->ev_dl[part], 0); };
    auto downloaded = [&](int part) { return cudaEventRecord(c->ev_dl[part], c->dl_stream); };
    if (out.host_cnt && staged_free(kOutSlabs)) return TDM_ECUDA;
    if (out.host_otf && staged_free(kOutSlabs + 1)) return TDM_ECUDA;
    // planes outside the cap band carry no hits and no OTF support
    const size_t plane = (size_t)D * D, lo = (size_t)p.zmin * plane, hi = (size_t)(p.zmin + p.band) * plane;
    const size_t NT = (size_t)D * D * D;
    if (cnt) {
        cudaMemsetAsync(cnt, 0, lo * sizeof(uint32_t), st);
        cudaMemsetAsync(cnt + hi, 0, (NT - hi) * sizeof(uint32_t), st);
    }
    if (otf) {
        cudaMemsetAsync(otf, 0, lo, st);
        cudaMemsetAsync(otf + hi, 0, NT - hi, st);
    }
    cudaEventRecord(c->ev_stage[4], st);
    {
        Launch l(c, K_GATHER, st);
        k_gather_z<D><<<dim3(D / 32, D), kGZ * 32, sm_a, st>>>(rec.val, rec.z, posspec, n, p, b.tw, b.vol, cnt, otf,
                                                                 1);
    }
    cudaEventRecord(c->ev_stage[5], st);
    if (ev_gathered && cudaEventRecord(ev_gathered, st)) return TDM_ECUDA;
    if (out.host_cnt) {
        if (download_after(c, st, c->ev_out[kOutSlabs], out.host_cnt, cnt, NT * sizeof(uint32_t)) ||
            downloaded(kOutSlabs))
            return TDM_ECUDA;
    }
    if (out.host_otf) {
        if (download_after(c, st, c->ev_out[kOutSlabs + 1], out.host_otf, otf, NT) || downloaded(kOutSlabs + 1))
            return TDM_ECUDA;
    }
    {
        Launch l(c, K_YPASS, st);
        k_ypass<D, 1><<<dim3(D / P::B, D), P::NT, sm_p, st>>>(b.vol, b.tw);
    }
    // x pass by slabs of z blocks; a slab's planes are final once it has run
    const bool host_vol = out.host_re || out.host_im;
    const int zblocks = D / P::B, nslab = host_vol ? (zblocks < kOutSlabs ? zblocks : kOutSlabs) : 1;
    for (int sl = 0; sl < nslab; ++sl) {
        const int zb0 = sl * zblocks / nslab, zb1 = (sl + 1) * zblocks / nslab;
        if (host_vol && staged_free(sl)) return TDM_ECUDA;
        {
            Launch l(c, K_XPASS, st);
            k_xpass<D><<<dim3(zb1 - zb0, D), P::NT, sm_p, st>>>(b.vol, b.tw, p.out_scale, zb0, re, im);
        }
        if (host_vol) {
            const size_t off = (size_t)zb0 * P::B * D * D, len = (size_t)(zb1 - zb0) * P::B * D * D;
            if (cudaEventRecord(c->ev_out[sl], st) || cudaStreamWaitEvent(c->dl_stream, c->ev_out[sl], 0))
                return TDM_ECUDA;
            if (out.host_re && cudaMemcpyAsync(out.host_re + off, re + off, len * sizeof(float),
                                               cudaMemcpyDeviceToHost, c->dl_stream))
                return TDM_ECUDA;
            if (out.host_im && cudaMemcpyAsync(out.host_im + off, im + off, len * sizeof(float),
                                               cudaMemcpyDeviceToHost, c->dl_stream))
                return TDM_ECUDA;
            if (downloaded(sl)) return TDM_ECUDA;
        }
    }
    cudaEventRecord(c->ev_stage[6], st);
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

template <int D>
int forward_impl(tdm_ctx* c, const float* xn, const float* xk, int n, float2* caps, const float2* data, CapRecs res,
                 double* misfit) {
    using P = PassCfg<D>;
    Buffers& b = c->b;
    const Params& p = c->p;
    const size_t sm_p = P::SMEM;
    if (allow_smem(k_fxpass<D>, sm_p) || allow_smem(k_ypass<D, -1>, sm_p) || allow_smem(k_fzpass<D>, sm_p))
        return TDM_ECUDA;
    const float scale = (float)(1.0 / ((double)p.out_scale * (double)D * D * D));
    {
        Launch l(c, K_XPASS);
        k_fxpass<D><<<dim3(D / P::B, D), P::NT, sm_p, c->stream>>>(xn, xk, b.tw, scale, b.vol);
    }
    {
        Launch l(c, K_YPASS);
        k_ypass<D, -1><<<dim3(D / P::B, D), P::NT, sm_p, c->stream>>>(b.vol, b.tw);
    }
    {
        Launch l(c, K_ZPASS);
        k_fzpass<D><<<dim3(D * D / P::B), P::NT, sm_p, c->stream>>>(b.vol, b.tw, p.zmin, p.band);
    }
    {
        Launch l(c, K_CAP_COLS);
        const int per = (p.F * p.F + 255) / 256;
        k_cap_sample<<<dim3(per < 16 ? per : 16, n), 256, 0, c->stream>>>(b.vol, b.posspec, p, b.s_tab, b.s_tabf, data,
                                                                          caps, res.val, res.z, misfit, b.err);
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

template <int D>
int adjoint_impl(tdm_ctx* c, CapRecs recs, int n, float* xn, float* xk, bool normalize) {
    using P = PassCfg<D>;
    Buffers& b = c->b;
    const Params& p = c->p;
    const size_t sm_a = GatherZ<D>::smem(p.band, n);
    const size_t sm_p = P::SMEM;
    if (sm_a > kMaxSmemPerCta) return TDM_EUNSUPPORTED;
    if (allow_smem(k_gather_z<D>, sm_a) || allow_smem(k_ypass<D, 1>, sm_p) || allow_smem(k_xpass<D>, sm_p))
        return TDM_ECUDA;
    {
        Launch l(c, K_GATHER);
        k_gather_z<D><<<dim3(D / 32, D), kGZ * 32, sm_a, c->stream>>>(recs.val, recs.z, b.posspec, n, p, b.tw, b.vol,
                                                                        nullptr, nullptr, normalize ? 1 : 0);
    }
    {
        Launch l(c, K_YPASS);
        k_ypass<D, 1><<<dim3(D / P::B, D), P::NT, sm_p, c->stream>>>(b.vol, b.tw);
    }
    const float scale = normalize ? p.out_scale : (float)(1.0 / ((double)p.out_scale * (double)D * D * D));
    {
        Launch l(c, K_XPASS);
        k_xpass<D><<<dim3(D / P::B, D), P::NT, sm_p, c->stream>>>(b.vol, b.tw, scale, 0, xn, xk);
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

}  // namespace

// Dynamic shared memory of k_gather_z: per warp the sums and counts of its
// column group (or their exchange buffers), its plane owners and a 32-lane
// staging row; the CTA's OTF bits and its list of n angles at most.
size_t gather_smem_bytes(int D, int band, int n) {
    switch (D) {
        case 128: return GatherZ<128>::smem(band, n);
        case 256: return GatherZ<256>::smem(band, n);
        case 512: return GatherZ<512>::smem(band, n);
        default: return GatherZ<1024>::smem(band, n);
    }
}

int launch_cap(tdm_ctx* c, int a0, int n, bool form) {
    if (c->p.F & (c->p.F - 1)) return launch_cap_generic(c, a0, n, form);
    switch (c->p.F) {
        case 64: return cap_impl<64>(c, a0, n, form);
        case 128: return cap_impl<128>(c, a0, n, form);
        case 256: return cap_impl<256>(c, a0, n, form);
        case 512: return cap_impl<512>(c, a0, n, form);
        default: return TDM_EUNSUPPORTED;
    }
}

int launch_volume(tdm_ctx* c, int n, const VolumeOut& out, cudaStream_t st, CapRecs rec, const int2* posspec,
                  cudaEvent_t ev_gathered) {
    switch (c->p.D) {
        case 128: return volume_impl<128>(c, n, out, st, rec, posspec, ev_gathered);
        case 256: return volume_impl<256>(c, n, out, st, rec, posspec, ev_gathered);
        case 512: return volume_impl<512>(c, n, out, st, rec, posspec, ev_gathered);
        case 1024: return volume_impl<1024>(c, n, out, st, rec, posspec, ev_gathered);
        default: return TDM_EUNSUPPORTED;
    }
}

int launch_forward(tdm_ctx* c, const float* xn, const float* xk, int n, float2* caps, const float2* data,
                   CapRecs res, double* misfit) {
    switch (c->p.D) {
        case 128: return forward_impl<128>(c, xn, xk, n, caps, data, res, misfit);
        case 256: return forward_impl<256>(c, xn, xk, n, caps, data, res, misfit);
        case 512: return forward_impl<512>(c, xn, xk, n, caps, data, res, misfit);
        case 1024: return forward_impl<1024>(c, xn, xk, n, caps, data, res, misfit);
        default: return TDM_EUNSUPPORTED;
    }
}

int launch_adjoint(tdm_ctx* c, CapRecs recs, int n, float* xn, float* xk, bool normalize) {
    switch (c->p.D) {
        case 128: return adjoint_impl<128>(c, recs, n, xn, xk, normalize);
        case 256: return adjoint_impl<256>(c, recs, n, xn, xk, normalize);
        case 512: return adjoint_impl<512>(c, recs, n, xn, xk, normalize);
        case 1024: return adjoint_impl<1024>(c, recs, n, xn, xk, normalize);
        default: return TDM_EUNSUPPORTED;
    }
}

int launch_cap_pack(tdm_ctx* c, const float2* caps, int n, CapRecs recs) {
    const int per = (c->p.F * c->p.F + 255) / 256;
    {
        Launch l(c, K_CAP_COLS);
        k_cap_pack<<<dim3(per < 16 ? per : 16, n), 256, 0, c->stream>>>(caps, c->b.posspec, c->p, c->b.s_tab,
                                                                        c->b.s_tabf, recs.val, recs.z, c->b.err);
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

int launch_tv_step(tdm_ctx* c, const float* xn, const float* xk, const float* gn, const float* gk, float step,
                   float tv_n, float tv_k, float eps, float nlo, float nhi, float klo, float khi, float* xn_out,
                   float* xk_out) {
    const int D = c->p.D;
    {
        Launch l(c, K_FORM);
        k_tv_step<<<152 * 8, 256, 0, c->stream>>>(xn, xk, gn, gk, D, step, tv_n, tv_k, eps * eps, nlo, nhi, klo, khi,
                                                   xn_out, xk_out);
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

}  // namespace tdm
