// Herraez phase unwrapping (VOLKOV 0): phaseUnwrapping_Mat,
// pretraitement_hors_axe_CPU/deroulement_herraez.cpp:32-74, as
// pretraitement_hors_axe_CPU/main.cpp:262-266 calls it on each angle's wrapped
// phase.  The result is the reference's bit for bit, given the same float
// wrapped phase:
//
//  k_hz_reliability  initialisePIXELs and calculate_reliability (:333-413):
//                    second differences of the wrapped phase in float for the
//                    interior; border pixels keep 9999999 + rand() (an int sum
//                    that wraps past INT_MAX), from the C library's generator
//                    as the reference's loop draws it: F^2 draws per earlier
//                    angle (host table, crand_border_table).
//  k_hz_edges        horizentalEDGEs, verticalEDGEs (:415-459): each edge's
//                    reliability (the two pixels' sum) and its 2 pi jump.
//  k_hz_sort_level   quick_sort (:163-213): the reference's merge sort on edge
//                    indices, which halves with size/2 so that the last index
//                    of an odd-sized run stays where it is; the later merges
//                    then see runs that are not sorted.  Mix (:113-159) merges
//                    them by comparing heads, which interleaves two runs as a
//                    stable merge of their prefix maxima does, so each element
//                    carries its run's prefix maximum: merging leaves it
//                    unchanged, and an odd node's leftover takes the maximum
//                    of its node when it joins its parent's run.  One launch
//                    per recursion depth, deepest first; every node of a depth
//                    has the same size.  Each element of a node's two halves
//                    finds its place by a binary search on the other half's
//                    prefix maxima (ties: the first half first, as in Mix).
//  k_hz_gather       gatherPIXELs and unwrapImage (:461-575), one CTA per
//                    angle: the edges in sorted order merge pixel groups.
//                    The reference keeps each group as a linked list and adds
//                    the merged group's 2 pi offset to every member; here the
//                    groups are a union-find forest in shared memory whose
//                    links carry the 2 pi offset to the parent (int8; -128
//                    marks a root, whose parent slot holds the group's size),
//                    and which
//                    takes the same decisions (a lone pixel 2 joins pixel 1's
//                    group, else a lone pixel 1 joins pixel 2's, else the
//                    larger group absorbs the other, ties to group 2), so each
//                    pixel's count is the reference's.  One thread merges;
//                    its warp fetches the next 32 sorted edges meanwhile.
#include "tdm_internal.cuh"

namespace tdm {
namespace {

constexpr float kHzPi = 3.141592654f, kHzTwoPi = 6.283185307f;  // deroulement_herraez.cpp:9-10
constexpr int kHzThreads = 256;

__device__ __forceinline__ float hz_wrap(float v) {  // wrap (:357-365)
    return v > kHzPi ? __fsub_rn(v, kHzTwoPi) : (v < -kHzPi ? __fadd_rn(v, kHzTwoPi) : v);
}

// Pixels of edge e: the F (F - 1) horizontal edges row by row, then the
// (F - 1) F vertical ones.
__device__ __forceinline__ void hz_edge(int e, int F, int& p1, int& p2) {
    const int nh = F * (F - 1);
    if (e < nh) {
        const int i = e / (F - 1);
        p1 = e + i;
        p2 = p1 + 1;
    } else {
        p1 = e - nh;
        p2 = p1 + F;
    }
}

// An edge's payload through the sort: its first pixel, whether it is
// vertical, and its 2 pi jump + 1: (p1 << 3) | (vertical << 2) | (jump + 1).
__device__ __forceinline__ void hz_payload_pixels(uint32_t pl, int F, int& p1, int& p2) {
    p1 = (int)(pl >> 3);
    p2 = p1 + ((pl & 4u) ? F : 1);
}

__global__ void __launch_bounds__(kHzThreads)
k_hz_reliability(const float* __restrict__ phase, const int* __restrict__ border_rand, int a0, int F,
                 float* __restrict__ rel) {
    const int a = blockIdx.y, FF = F * F;
    const int p = blockIdx.x * kHzThreads + threadIdx.x;
    if (p >= FF) return;
    const float* ph = phase + (size_t)a * FF;
    const int i = p / F, j = p - i * F;
    float r;
    if (i == 0 || j == 0 || i == F - 1 || j == F - 1) {
        // border index: row 0, then columns 0 and F - 1 of rows 1 .. F - 2, then row F - 1
        const int b = i == 0 ? j : (i == F - 1 ? F + 2 * (F - 2) + j : F + 2 * (i - 1) + (j ? 1 : 0));
        const uint32_t v = 9999999u + (uint32_t)border_rand[(size_t)(a0 + a) * (4 * F - 4) + b];
        r = __int2float_rn((int)v);
    } else {
        const float c = ph[p];
        auto d2 = [&](int o) { return __fsub_rn(hz_wrap(__fsub_rn(ph[p - o], c)), hz_wrap(__fsub_rn(c, ph[p + o]))); };
        const float H = d2(1), V = d2(F), D1 = d2(F + 1), D2 = d2(F - 1);
        r = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(H, H), __fmul_rn(V, V)), __fmul_rn(D1, D1)), __fmul_rn(D2, D2));
    }
    rel[(size_t)a * FF + p] = r;
}

// Sort arrays of one angle: the keys (each element's run prefix maximum)
// and the payloads, ne each.  An edge's own key, needed only when it joins a
// run as an odd node's leftover, is recomputed from the two pixels'
// reliabilities.
struct SortBuf {
    float* eff;
    uint32_t* pay;
};

// Per edge: key = its reliability, and its payload (hz_payload_pixels).
// The chunk's angle i keeps its arrays at offset i * stride.
__global__ void __launch_bounds__(kHzThreads)
k_hz_edges(const float* __restrict__ phase, const float* __restrict__ rel, int F, size_t stride, SortBuf out) {
    const int a = blockIdx.y, FF = F * F, ne = 2 * F * (F - 1);
    const int e = blockIdx.x * kHzThreads + threadIdx.x;
    if (e >= ne) return;
    int p1, p2;
    hz_edge(e, F, p1, p2);
    const float* ph = phase + (size_t)a * FF;
    const float* rl = rel + (size_t)a * FF;
    const float d = __fsub_rn(ph[p1], ph[p2]);  // find_wrap (:368-380)
    const int jump = d > kHzPi ? -1 : (d < -kHzPi ? 1 : 0);
    const size_t o = a * stride + e;
    out.eff[o] = __fadd_rn(rl[p1], rl[p2]);  // a run of one
    out.pay[o] = ((uint32_t)p1 << 3) | (p2 - p1 == 1 ? 0u : 4u) | (uint32_t)(jump + 1);
}

struct SortLevel {
    int ne, depth;
};

// Depth `depth` of the sort: the node (s, n) of that depth holding element i
// merges its halves [s, s + h) and [s + h, s + 2h), h = n / 2, which the
// deeper launches merged; everything else keeps its place.
__global__ void __launch_bounds__(kHzThreads)
k_hz_sort_level(SortBuf in, SortBuf out, size_t stride, const float* __restrict__ rel, int F, SortLevel L) {
    const int i = blockIdx.x * kHzThreads + threadIdx.x;
    if (i >= L.ne) return;
    const size_t base = blockIdx.y * stride;
    const float* k = in.eff + base;
    int s = 0, n = L.ne;
    bool inside = true;
    for (int d = 0; d < L.depth; ++d) {
        const int h = n / 2;
        if (i < s + h) {
            n = h;
        } else if (i < s + 2 * h) {
            s += h;
            n = h;
        } else {
            inside = false;  // the leftover of an odd-sized ancestor
            break;
        }
    }
    const uint32_t pl = in.pay[base + i];
    float x = k[i];
    int dst = i;
    const int h = n / 2;
    if (inside && h >= 1 && i < s + 2 * h) {
        if (i < s + h) {  // first half: after the second half's elements strictly below x
            int lo = 0, hi = h;
            while (lo < hi) {
                const int m = (lo + hi) >> 1;
                if (k[s + h + m] < x) lo = m + 1;
                else hi = m;
            }
            dst = i + lo;
        } else {  // second half: after the first half's elements up to x
            int lo = 0, hi = h;
            while (lo < hi) {
                const int m = (lo + hi) >> 1;
                if (k[s + m] <= x) lo = m + 1;
                else hi = m;
            }
            dst = i - h + lo;
        }
    } else if (inside && h >= 1 && (n & 1)) {  // the odd node's leftover joins the node's run at its end
        int p1, p2;
        hz_payload_pixels(pl, F, p1, p2);
        const float* rl = rel + (size_t)blockIdx.y * F * F;
        x = fmaxf(fmaxf(k[s + h - 1], k[s + 2 * h - 1]), __fadd_rn(rl[p1], rl[p2]));
    }
    out.eff[base + dst] = x;
    out.pay[base + dst] = pl;
}

// The forest of k_hz_gather for F x F pixels: per pixel the parent (or, at a
// root, the group's size - 1) and the 2 pi offset to the parent as int8,
// kHzRoot marking a root.  In shared memory (uint16 parents) up to 256^2
// pixels: 3 bytes a pixel.
constexpr int kHzRoot = -128;
size_t hz_gather_smem(int F) {
    const size_t n = (size_t)F * F;
    return n * 3;
}

// One CTA per angle.  Idx is the parent's type: uint16_t with the forest in
// shared memory (up to 256^2 pixels), uint32_t with it in global memory
// (forest, up to n parents then n offsets, one per angle at a stride).
template <class Idx, bool SHARED>
__global__ void __launch_bounds__(kHzThreads)
k_hz_gather(const uint32_t* __restrict__ pays, size_t stride, const float* __restrict__ phase, int F,
            float* __restrict__ unwrapped, int* __restrict__ err, unsigned char* __restrict__ forest,
            size_t forest_stride) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int a = blockIdx.x, n = F * F, ne = 2 * F * (F - 1);
    unsigned char* base = SHARED ? smraw : forest + a * forest_stride;
    Idx* up = reinterpret_cast<Idx*>(base);
    int8_t* pot = reinterpret_cast<int8_t*>(up + n);
    __shared__ uint32_t batch[32];
    for (int p = threadIdx.x; p < n; p += kHzThreads) {
        up[p] = 0;  // every pixel the root of its own group of size 1
        pot[p] = (int8_t)kHzRoot;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const uint32_t* ps = pays + a * stride;
        uint32_t nxt = lane < ne ? ps[lane] : 0u;
        int bad = 0;
        // root of pixel p and p's 2 pi count relative to it, halving the path
        // (each visited pixel is relinked to its grandparent)
        auto find = [&](int p, int& acc) {
            acc = 0;
            int pp = pot[p];
            if (pp == kHzRoot) return p;
            int q = (int)up[p];
            while (true) {
                const int pq = pot[q];
                if (pq == kHzRoot) {
                    acc += pp;
                    return q;
                }
                const int g = (int)up[q];
                const int v = pp + pq;  // p's offset to g
                bad |= v < -127 || v > 127;
                pot[p] = (int8_t)v;
                up[p] = (Idx)g;
                acc += v;
                p = g;
                pp = pot[g];
                if (pp == kHzRoot) return g;
                q = (int)up[g];
            }
        };
        for (int k0 = 0; k0 < ne; k0 += 32) {
            batch[lane] = nxt;
            nxt = k0 + 32 + lane < ne ? ps[k0 + 32 + lane] : 0u;  // the next batch, in flight meanwhile
            __syncwarp();
            if (lane == 0) {
                const int cnt = min(32, ne - k0);
                for (int t = 0; t < cnt; ++t) {
                    const uint32_t pl = batch[t];
                    const int jump = (int)(pl & 3u) - 1;
                    int p1, p2;
                    hz_payload_pixels(pl, F, p1, p2);
                    int a1, a2;
                    const int r1 = find(p1, a1), r2 = find(p2, a2);
                    if (r1 == r2) continue;
                    const int s1 = (int)up[r1] + 1, s2 = (int)up[r2] + 1;
                    // child root c joins parent root r with 2 pi offset v; the group has `size` pixels
                    auto link = [&](int c, int r, int v, int size) {
                        bad |= v < -127 || v > 127;
                        up[c] = (Idx)r;
                        pot[c] = (int8_t)v;
                        up[r] = (Idx)(size - 1);
                    };
                    if (s2 == 1) link(r2, r1, a1 - jump, s1 + 1);              // pixel 2 alone
                    else if (s1 == 1) link(r1, r2, a2 + jump, s2 + 1);         // pixel 1 alone
                    else if (s1 > s2) link(r2, r1, a1 - jump - a2, s1 + s2);   // group 2 into group 1
                    else link(r1, r2, a2 + jump - a1, s1 + s2);                // group 1 into group 2
                }
            }
            __syncwarp();
        }
        if (lane == 0 && bad) atomicOr(err, 8);
        if (!SHARED) __threadfence_block();
    }
    __syncthreads();
    const float* ph = phase + (size_t)a * n;
    float* out = unwrapped + (size_t)a * n;
    for (int p = threadIdx.x; p < n; p += kHzThreads) {
        int acc = 0;
        for (int q = p; pot[q] != kHzRoot; q = (int)up[q]) acc += pot[q];
        out[p] = __fadd_rn(ph[p], __fmul_rn(kHzTwoPi, __int2float_rn(acc)));
    }
}

}  // namespace

size_t herraez_gather_smem(int F) { return hz_gather_smem(F); }

// The m angles of the chunk starting at stack angle a0: b.phase -> b.unwrapped,
// with b.gx (reliabilities) and b.qc / b.tq (keys and payloads, ping-pong) as
// scratch.
int launch_herraez(tdm_ctx* c, int a0, int m) {
    Buffers& b = c->b;
    const int F = c->p.F, FF = F * F, ne = 2 * F * (F - 1);
    const size_t stride = (size_t)c->p.L * F * 2;  // floats per angle in qc and tq (L F complex >= 2 ne)
    SortBuf buf[2];
    float* base[2] = {reinterpret_cast<float*>(b.qc), reinterpret_cast<float*>(b.tq)};
    for (int k = 0; k < 2; ++k) buf[k] = SortBuf{base[k], reinterpret_cast<uint32_t*>(base[k] + ne)};
    const size_t smem = hz_gather_smem(F);
    const bool shared = F <= 256 && smem <= kMaxSmemPerCta;  // uint16 parents
    if (!b.hz_rand) return TDM_EUNSUPPORTED;
    if (shared && max_dynamic_smem(reinterpret_cast<const void*>(k_hz_gather<uint16_t, true>), smem) != cudaSuccess)
        return TDM_ECUDA;
    {
        Launch l(c, K_HERRAEZ);
        k_hz_reliability<<<dim3((FF + kHzThreads - 1) / kHzThreads, m), kHzThreads, 0, c->stream>>>(
            b.phase, b.hz_rand, a0, F, b.gx);
    }
    {
        Launch l(c, K_HERRAEZ);
        k_hz_edges<<<dim3((ne + kHzThreads - 1) / kHzThreads, m), kHzThreads, 0, c->stream>>>(b.phase, b.gx, F,
                                                                                             stride, buf[0]);
    }
    // depths whose nodes have at least 2 elements, deepest first
    int depth = 0;
    for (int n = ne; n / 2 >= 2; n /= 2) ++depth;
    int cur = 0;
    for (int d = depth; d >= 0; --d, cur ^= 1) {
        Launch l(c, K_HERRAEZ);
        k_hz_sort_level<<<dim3((ne + kHzThreads - 1) / kHzThreads, m), kHzThreads, 0, c->stream>>>(
            buf[cur], buf[cur ^ 1], stride, b.gx, F, SortLevel{ne, d});
    }
    if (shared) {
        Launch l(c, K_HERRAEZ);
        k_hz_gather<uint16_t, true><<<m, kHzThreads, smem, c->stream>>>(buf[cur].pay, stride, b.phase, F,
                                                                         b.unwrapped, b.err, nullptr, 0);
    } else {  // the forest in the other sort buffer, free now: 5 bytes a pixel within 16 F^2 an angle
        Launch l(c, K_HERRAEZ);
        k_hz_gather<uint32_t, false><<<m, kHzThreads, 0, c->stream>>>(
            buf[cur].pay, stride, b.phase, F, b.unwrapped, b.err, reinterpret_cast<unsigned char*>(base[cur ^ 1]),
            stride * sizeof(float));
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

}  // namespace tdm
