// C ABI of the reconstruction path: context, tables, buffers and entry points.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "bulk_copy.cuh"
#include "host_tables.h"
#include "tdm_internal.cuh"

using namespace tdm;

namespace tdm {
const char* const kKernelNames[K_COUNT] = {
    "extract_rows", "extract_cols", "argmax", "field_rows", "field_cols", "volkov_rows", "volkov_cols",
    "volkov_integ_rows", "volkov_integ_cols", "aber_fit", "form", "cap_rows", "cap_cols", "gather",
    "ypass", "xpass", "posspec", "zpass", "herraez"};

cudaEvent_t prof_event(tdm_ctx* c) {
    if (!c->ev_pool.empty()) {
        cudaEvent_t e = c->ev_pool.back();
        c->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

cudaError_t max_dynamic_smem(const void* fn, size_t bytes) {
    int dev = 0;
    if (cudaError_t e = cudaGetDevice(&dev)) return e;
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> done;  // largest size set per kernel and device
    std::lock_guard<std::mutex> lk(mu);
    size_t& have = done[{fn, dev}];
    if (have >= bytes) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) have = bytes;
    return e;
}
}  // namespace tdm

namespace {

void prof_release(tdm_ctx* c) {
    for (const ProfRec& r : c->prof_recs) {
        c->ev_pool.push_back(r.a);
        c->ev_pool.push_back(r.b);
    }
    c->prof_recs.clear();
}

int fail(tdm_ctx* c, int code, const std::string& msg) {
    if (c) c->last_error = msg;
    return code;
}

int cuda_fail(tdm_ctx* c, cudaError_t e, const char* what) {
    if (c) c->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? TDM_ENOMEM : TDM_ECUDA;
}

#define TDM_CU(call)                                                   \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #call);         \
    } while (0)

bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }


bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

template <class T>
int dev_alloc(tdm_ctx* c, T** p, size_t count) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
    return TDM_OK;
}

void free_all(tdm_ctx* c) {
    Buffers& b = c->b;
    void* ptrs[] = {b.tw, b.win_h, b.tuk_f, b.s_tab, b.s_tabf, b.wq, b.holo_stage, b.inter, b.spectra, b.posspec,
                    b.specval, b.argpart, b.I1, b.phase, b.amp, b.zph, b.gx, b.qc, b.tq, b.phase_sum, b.unwrapped, b.beta,
                    b.fit_part, b.fit_done, b.fields, b.r1, b.rec_buf[0].val, b.rec_buf[0].z, b.rec_buf[1].val,
                    b.rec_buf[1].z, b.posspec_vol[0], b.posspec_vol[1], b.vol, b.out_re, b.out_im, b.out_otf,
                    b.out_cnt, b.samp_idx, b.samp_q, b.rinv, b.err, b.xv[0], b.xv[1], b.xv[2], b.xv[3],
                    b.xv[4], b.xv[5], b.caps, b.rec2.val, b.rec2.z, b.misfit, b.ref_inv, b.hz_rand};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    b = Buffers{};
}

__global__ void k_pack_posspec(const int32_t* __restrict__ xy, int n, int2* __restrict__ out) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < n) out[a] = make_int2(xy[a], xy[n + a]);
}
__global__ void k_unpack_posspec(const int2* __restrict__ in, int n, int32_t* __restrict__ xy) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < n) {
        xy[a] = in[a].x;
        xy[n + a] = in[a].y;
    }
}

// Aberration sample points and an orthonormal basis of the degree-4
// polynomials over them (modified Gram-Schmidt in long double, twice).
int build_aberration(tdm_ctx* c, const uint8_t* mask_host) {
    const int F = c->p.F;
    std::vector<int> idx;
    std::vector<long double> A;  // nsamp x kNC
    const long double h = 0.5L * (F - 1);
    // countM (Correction_aberration.cpp:86-106) marks every 5th row/column
    // pixel with value > 45; the samples are those pixels in row-major order.
    for (int y = 0; y < F; ++y)
        for (int x = 0; x < F; ++x) {
            const uint8_t v = mask_host ? mask_host[(size_t)y * F + x] : 255;
            if (x % 5 == 0 && y % 5 == 0 && v > 45) {
                idx.push_back(y * F + x);
                const long double u = (x - h) / h, w = (y - h) / h;
                for (int px = 0; px <= 4; ++px)
                    for (int py = 0; px + py <= 4; ++py) A.push_back(std::pow(u, (long double)px) * std::pow(w, (long double)py));
            }
        }
    const int ns = (int)idx.size();
    if (ns < kNC) return fail(c, TDM_EDATA, "aberration mask leaves fewer than 15 background samples");
    std::vector<long double> Q(A), R(kNC * kNC, 0.0L);
    for (int k = 0; k < kNC; ++k) {
        for (int pass = 0; pass < 2; ++pass)
            for (int i = 0; i < k; ++i) {
                long double d = 0;
                for (int s = 0; s < ns; ++s) d += Q[(size_t)s * kNC + i] * Q[(size_t)s * kNC + k];
                R[i * kNC + k] += d;
                for (int s = 0; s < ns; ++s) Q[(size_t)s * kNC + k] -= d * Q[(size_t)s * kNC + i];
            }
        long double nrm = 0;
        for (int s = 0; s < ns; ++s) nrm += Q[(size_t)s * kNC + k] * Q[(size_t)s * kNC + k];
        nrm = std::sqrt(nrm);
        if (!(nrm > 1e-12L)) return fail(c, TDM_EDATA, "aberration samples do not determine a degree-4 fit");
        R[k * kNC + k] = nrm;
        for (int s = 0; s < ns; ++s) Q[(size_t)s * kNC + k] /= nrm;
    }
    // Rinv = R^-1 (upper triangular)
    std::vector<long double> Ri(kNC * kNC, 0.0L);
    for (int col = 0; col < kNC; ++col) {
        for (int row = col; row >= 0; --row) {
            long double s = (row == col) ? 1.0L : 0.0L;
            for (int k = row + 1; k <= col; ++k) s -= R[row * kNC + k] * Ri[k * kNC + col];
            Ri[row * kNC + col] = s / R[row * kNC + row];
        }
    }
    std::vector<float> qf((size_t)ns * kNC);
    for (size_t i = 0; i < qf.size(); ++i) qf[i] = (float)Q[i];
    std::vector<double> rd(kNC * kNC);
    for (int i = 0; i < kNC * kNC; ++i) rd[i] = (double)Ri[i];
    Buffers& b = c->b;
    if (b.samp_idx) cudaFree(b.samp_idx);
    if (b.samp_q) cudaFree(b.samp_q);
    b.samp_idx = nullptr;
    b.samp_q = nullptr;
    if (int rc = dev_alloc(c, &b.samp_idx, ns)) return rc;
    if (int rc = dev_alloc(c, &b.samp_q, qf.size())) return rc;
    TDM_CU(cudaMemcpy(b.samp_idx, idx.data(), ns * sizeof(int), cudaMemcpyHostToDevice));
    TDM_CU(cudaMemcpy(b.samp_q, qf.data(), qf.size() * sizeof(float), cudaMemcpyHostToDevice));
    TDM_CU(cudaMemcpy(b.rinv, rd.data(), rd.size() * sizeof(double), cudaMemcpyHostToDevice));
    c->nsamp = ns;
    return TDM_OK;
}

int check_geom(const tdm_geom* g, std::string& why) {
    if (!is_pow2(g->ccd_roix) || g->ccd_roix < 256 || g->ccd_roix > 2048) {
        why = "CCD_ROIX must be a power of two in [256, 2048]";
        return TDM_EUNSUPPORTED;
    }
    const int F = 2 * g->nxmax;
    if (!((is_pow2(F) && F >= 64 && F <= 512) || generic_field_size(F))) {
        why = "2*NXMAX must be a power of two in [64, 512] or 250";
        return TDM_EUNSUPPORTED;
    }
    if (!is_pow2(g->dim_final) || g->dim_final < 4 * g->nxmax || g->dim_final > 1024 || g->dim_final < 128) {
        why = "DIM_FINAL must be a power of two in [max(128, 4*NXMAX), 1024]";
        return TDM_EUNSUPPORTED;
    }
    const int x0 = g->circle_cx - g->nxmax, y0 = g->circle_cy - g->nxmax;
    if (x0 < 0 || y0 < 0 || x0 + F > g->ccd_roix || y0 + F > g->ccd_roix) {
        why = "crop window (CIRCLE_CX/CY +- NXMAX) outside the hologram spectrum";
        return TDM_EINVAL;
    }
    if (!(g->na > 0) || !(g->n0 > 0) || !(g->lambda0 > 0) || !(g->f_obj > 0) || !(g->rf > 0) || !(g->f_tube > 0) ||
        !(g->tpcam > 0)) {
        why = "optical parameters must be positive";
        return TDM_EINVAL;
    }
    return TDM_OK;
}

}  // namespace

extern "C" {

int tdm_derive(const tdm_geom* g, tdm_derived* d) {
    if (!g || !d) return TDM_EINVAL;
    // manip (pretraitement_hors_axe_CPU/manip.cpp:35-57,104; Reconstruction/src/manip.cpp:56-94)
    const double G = g->f_tube / g->f_obj;
    const double Gt = G / g->rf;
    d->tp_holo = g->tpcam / Gt;
    const size_t twoN = 2 * (size_t)g->nxmax;
    d->tp_uborn = d->tp_holo * g->ccd_roix / (double)twoN;
    d->delta_f = 1 / (d->tp_uborn * 2 * (double)g->nxmax);
    d->tp_tomo = d->tp_uborn * (double)twoN / (double)g->dim_final;
    d->rayon = std::round((double)(size_t)g->nxmax * g->n0 / g->na);
    return TDM_OK;
}

int tdm_create(const tdm_geom* geom, int max_angles, tdm_ctx** out) {
    if (!geom || !out || max_angles <= 0) return TDM_EINVAL;
    *out = nullptr;
    if (max_angles > 65535) {  // a voxel's hit count is kept in 16 bits while its column is gathered
        fprintf(stderr, "tdm_create: at most 65535 angles per stack\n");
        return TDM_EUNSUPPORTED;
    }
    std::string why;
    if (int rc = check_geom(geom, why)) {
        fprintf(stderr, "tdm_create: %s\n", why.c_str());
        return rc;
    }
    tdm_ctx* c = new tdm_ctx();
    c->g = *geom;
    c->max_angles = max_angles;
    c->chunk_cap = std::min(kChunkCapMax, (max_angles + 15) / 16 * 16);
    tdm_derive(geom, &c->dv);
    Params& p = c->p;
    p.H = geom->ccd_roix;
    p.N = geom->nxmax;
    p.F = 2 * p.N;
    p.L = 2 * p.F;
    p.D = geom->dim_final;
    p.x0 = geom->circle_cx - p.N;
    p.y0 = geom->circle_cy - p.N;
    p.born = geom->born ? 1 : 0;
    p.c_aber = geom->c_aber ? 1 : 0;
    p.deroul = geom->deroul ? 1 : 0;
    p.volkov = geom->volkov ? 1 : 0;
    p.rayon = c->dv.rayon;
    p.inv_rayon = 1.0 / c->dv.rayon;
    const int N = p.N, F = p.F, D = p.D;
    // disc test fd^2 < COEF_NA_OBJ_LIMIT * N^2 on integers (fonctions.cpp:915)
    const double lim = geom->coef_na_obj_limit * (double)(N * N);
    p.disc_thr = (int)std::min<double>(std::ceil(lim), 2.0 * N * N + 1);
    // cap heights sqrt(rayon^2 - fd^2) exactly as fonctions.cpp:920, and the z band
    const double r2 = p.rayon * p.rayon;
    // rayon is an integer: below 2^24, rayon^2 - fd^2 is an exact float and
    // its correctly rounded float sqrt equals (float)sqrt in double (checked
    // for every integer below 2^24), so the kernels compute the float table
    p.r2i = r2 < 16777216.0 ? (int)r2 : 0;
    std::vector<double> stab((size_t)F * F, std::numeric_limits<double>::quiet_NaN());
    double smin = std::numeric_limits<double>::infinity();
    for (int fdy = -N; fdy < N; ++fdy)
        for (int fdx = -N; fdx < N; ++fdx) {
            const double fdz2 = r2 - fdx * fdx - fdy * fdy;
            stab[(size_t)(fdy + N) * F + fdx + N] = std::sqrt(fdz2);
            if (fdx * fdx + fdy * fdy < p.disc_thr) {
                if (!(fdz2 >= 0)) {
                    delete c;
                    fprintf(stderr, "tdm_create: NA disc reaches beyond the Ewald sphere\n");
                    return TDM_EUNSUPPORTED;
                }
                smin = std::min(smin, std::sqrt(fdz2));
            }
        }
    double fzmin = std::numeric_limits<double>::infinity(), fzmax = 0;
    for (int fy = -N; fy < N; ++fy)
        for (int fx = -N; fx < N; ++fx) {
            const double cz = r2 - fx * fx - fy * fy;
            if (std::round(cz) >= 0) {
                fzmin = std::min(fzmin, std::sqrt(cz));
                fzmax = std::max(fzmax, std::sqrt(cz));
            }
        }
    const int kmin = (int)std::round(smin - fzmax), kmax = (int)std::round(p.rayon - fzmin);
    p.zmin = D / 2 + kmin;
    p.band = kmax - kmin + 1;
    if (p.zmin < 0 || p.zmin + p.band > D) {
        delete c;
        fprintf(stderr, "tdm_create: Ewald caps exceed the DIM_FINAL volume along z\n");
        return TDM_EUNSUPPORTED;
    }
    if (gather_smem_bytes(D, p.band, max_angles) > kMaxSmemPerCta) {
        // the gather keeps each CTA's list of angles in shared memory
        int most = 0;
        while (gather_smem_bytes(D, p.band, most + 1) <= kMaxSmemPerCta) ++most;
        delete c;
        fprintf(stderr, "tdm_create: at most %d angles for this geometry (the cap gather's angle list of a "
                        "%d-plane cap band must fit one CTA's shared memory)\n", most, p.band);
        return TDM_EUNSUPPORTED;
    }
    // retroPropag_Born constants (Reconstruction/src/fonctions.cpp:885-902): k0 is a
    // float, and that file defines PI as 3.14159 (:2), which the cap weight keeps
    const double pi_ref = 3.14159;
    const float n0f = (float)geom->n0;
    const float kv = (float)(2 * pi_ref / geom->lambda0);
    const float k0 = kv * n0f;
    p.cap_scale = (float)(((double)k0 / pi_ref) * (-2 * pi_ref));
    p.dx2 = (float)std::pow(c->dv.tp_uborn, 2);
    const double k_v = 2 * M_PI / geom->lambda0;  // main.cpp:346-347
    p.out_scale = (float)(std::pow(c->dv.delta_f, 3) * (-1 / (2 * geom->n0 * k_v * k_v)));

    int rc = TDM_OK;
#define TRY(x)                         \
    do {                               \
        if ((rc = (x)) != TDM_OK) {    \
            free_all(c);               \
            tdm_ctx* dead = c;         \
            std::string m = dead->last_error; \
            delete dead;               \
            fprintf(stderr, "tdm_create: %s\n", m.c_str()); \
            return rc;                 \
        }                              \
    } while (0)
    cudaGetDevice(&c->device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->dl_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->vol_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_lane_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_angles, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_vol_last, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_rec_free[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_rec_free[1], cudaEventDisableTiming) != cudaSuccess) {
        delete c;
        return TDM_ECUDA;
    }
    for (int i = 0; i < kMaxLanes - 1; ++i)
        if (cudaStreamCreateWithFlags(&c->lane_stream[i], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->ev_lane_join[i], cudaEventDisableTiming) != cudaSuccess) {
            tdm_destroy(c);
            return TDM_ECUDA;
        }
    for (int i = 0; i < kStageSlots; ++i) {
        cudaEventCreateWithFlags(&c->ev_copy[i], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&c->ev_free[i], cudaEventDisableTiming);
    }
    for (auto& e : c->ev_stage) cudaEventCreate(&e);
    for (auto& e : c->ev_out) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    for (auto& e : c->ev_dl) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    Buffers& b = c->b;
    const size_t FF = (size_t)F * F, M = max_angles, CH = c->chunk_cap, L = p.L;
    TRY(dev_alloc(c, &b.tw, kTwTotal));
    TRY(dev_alloc(c, &b.win_h, p.H));
    TRY(dev_alloc(c, &b.tuk_f, F));
    TRY(dev_alloc(c, &b.s_tab, FF));
    TRY(dev_alloc(c, &b.s_tabf, FF));
    TRY(dev_alloc(c, &b.wq, 4 * F));
    TRY(dev_alloc(c, &b.holo_stage, 2 * CH * p.H * p.H * 2));
    TRY(dev_alloc(c, &b.inter, CH * p.H * F));
    TRY(dev_alloc(c, &b.spectra, M * FF));
    TRY(dev_alloc(c, &b.posspec, M));
    TRY(dev_alloc(c, &b.specval, M));
    TRY(dev_alloc(c, &b.argpart, CH * kArgPartsMax));
    TRY(dev_alloc(c, &b.I1, CH * FF));
    TRY(dev_alloc(c, &b.phase, CH * FF));
    TRY(dev_alloc(c, &b.amp, CH * FF));
    TRY(dev_alloc(c, &b.zph, CH * FF));
    TRY(dev_alloc(c, &b.gx, CH * FF));
    TRY(dev_alloc(c, &b.qc, CH * L * F));
    TRY(dev_alloc(c, &b.tq, CH * L * F));
    TRY(dev_alloc(c, &b.phase_sum, CH * kPhaseParts));
    TRY(dev_alloc(c, &b.unwrapped, CH * FF));
    TRY(dev_alloc(c, &b.beta, CH * 2 * kNC));
    TRY(dev_alloc(c, &b.fit_part, CH * 2 * 8 * kNC));
    TRY(dev_alloc(c, &b.fit_done, CH * 2));
    TRY(dev_alloc(c, &b.fields, M * FF));
    TRY(dev_alloc(c, &b.r1, CH * FF));
    for (auto& r : b.rec_buf) {
        TRY(dev_alloc(c, &r.val, M * FF));
        TRY(dev_alloc(c, &r.z, M * FF));
    }
    TRY(dev_alloc(c, &b.posspec_vol[0], M));
    TRY(dev_alloc(c, &b.posspec_vol[1], M));
    b.rec = b.rec_buf[0];
    TRY(dev_alloc(c, &b.vol, (size_t)D * D * D));
    TRY(dev_alloc(c, &b.rinv, kNC * kNC));
    TRY(dev_alloc(c, &b.err, 4));
    // tables
    const std::vector<float2> tw = twiddle_table();
    const std::vector<float2> wh = hologram_window(p.H);
    std::vector<double> tf = tukey_factor(F, 0.1f);
    c->tuk_h_flat = tukey_flat(p.H, 0.05f);
    c->tuk_f_flat = tukey_flat(F, 0.1f);
    std::vector<float> tff(tf.begin(), tf.end());
    std::vector<float> stabf(stab.begin(), stab.end());
    std::vector<float2> wq(4 * F);  // exp(-2 pi i k / 4F), for the mixed-radix passes
    for (int k = 0; k < 4 * F; ++k) {
        const double ang = -2.0 * M_PI * (double)k / (4.0 * F);
        wq[k] = make_float2((float)std::cos(ang), (float)std::sin(ang));
    }
    if (cudaMemcpy(b.tw, tw.data(), kTwTotal * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b.win_h, wh.data(), p.H * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b.tuk_f, tff.data(), F * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b.s_tab, stab.data(), FF * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b.s_tabf, stabf.data(), FF * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b.wq, wq.data(), 4 * F * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(b.err, 0, 4 * sizeof(int)) != cudaSuccess ||
        cudaMemset(b.fit_done, 0, CH * 2 * sizeof(unsigned)) != cudaSuccess)
        TRY(cuda_fail(c, cudaGetLastError(), "table upload"));
    if (p.c_aber && p.deroul && !p.volkov) {  // Herraez unwrapping's border reliabilities
        // its merging runs one CTA per angle: twice as many angles in flight
        if (32 * c->lanes <= c->chunk_cap) c->chunk = c->holo_chunk = 32;
        const std::vector<int> br = crand_border_table(F, max_angles);
        TRY(dev_alloc(c, &b.hz_rand, br.size()));
        if (cudaMemcpy(b.hz_rand, br.data(), br.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
            TRY(cuda_fail(c, cudaGetLastError(), "table upload"));
    }
    if (p.c_aber) TRY(build_aberration(c, nullptr));
#undef TRY
    *out = c;
    return TDM_OK;
}

int tdm_destroy(tdm_ctx* c) {
    if (!c) return TDM_EINVAL;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    if (c->dl_stream) cudaStreamSynchronize(c->dl_stream);
    if (c->vol_stream) cudaStreamSynchronize(c->vol_stream);
    for (cudaStream_t l : c->lane_stream)
        if (l) cudaStreamSynchronize(l);
    free_all(c);
    for (int i = 0; i < kStageSlots; ++i) {
        if (c->ev_copy[i]) cudaEventDestroy(c->ev_copy[i]);
        if (c->ev_free[i]) cudaEventDestroy(c->ev_free[i]);
    }
    for (int i = 0; i < kMaxLanes - 1; ++i) {
        if (c->lane_stream[i]) cudaStreamDestroy(c->lane_stream[i]);
        if (c->ev_lane_join[i]) cudaEventDestroy(c->ev_lane_join[i]);
    }
    for (auto& e : c->ev_stage)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->ev_out)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->ev_dl)
        if (e) cudaEventDestroy(e);
    prof_release(c);
    for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->dl_stream) cudaStreamDestroy(c->dl_stream);
    if (c->vol_stream) cudaStreamDestroy(c->vol_stream);
    for (cudaEvent_t e : {c->ev_angles, c->ev_vol_last, c->ev_rec_free[0], c->ev_rec_free[1], c->ev_lane_fork})
        if (e) cudaEventDestroy(e);
    delete c;
    return TDM_OK;
}

const char* tdm_last_error(const tdm_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

int tdm_get_derived(const tdm_ctx* c, tdm_derived* out) {
    if (!c || !out) return TDM_EINVAL;
    *out = c->dv;
    return TDM_OK;
}

// Orders the context stream after the volume stages that tdm_pipeline queued
// on vol_stream (every entry point but tdm_pipeline starts with it).
static cudaError_t join_volume(tdm_ctx* c) { return cudaStreamWaitEvent(c->stream, c->ev_vol_last, 0); }

int tdm_join(tdm_ctx* c) {
    if (!c) return TDM_EINVAL;
    cudaSetDevice(c->device);
    TDM_CU(join_volume(c));
    return TDM_OK;
}

int tdm_set_mask(tdm_ctx* c, const uint8_t* mask) {
    if (!c) return TDM_EINVAL;
    cudaSetDevice(c->device);
    // the background-sample tables are replaced with blocking copies: no work may still use them
    if (int rc = tdm_synchronize(c)) return rc;
    if (!c->p.c_aber) return TDM_OK;
    std::vector<uint8_t> hm;
    if (mask && is_device_ptr(mask)) {
        hm.resize((size_t)c->p.F * c->p.F);
        TDM_CU(cudaMemcpy(hm.data(), mask, hm.size(), cudaMemcpyDeviceToHost));
        mask = hm.data();
    }
    TDM_CU(cudaStreamSynchronize(c->stream));
    return build_aberration(c, mask);
}

// initRef (fonctions.cpp:46-61): the reference amplitude is sqrt(I_ref), 1
// where I_ref is 0; kept as its float reciprocal (double arithmetic, one
// rounding), multiplied into each pixel by the extraction row pass.
int tdm_set_reference_intensity(tdm_ctx* c, const float* intensity) {
    if (!c) return TDM_EINVAL;
    cudaSetDevice(c->device);
    if (int rc = tdm_synchronize(c)) return rc;  // no queued extraction may still read the table
    if (!intensity) {
        c->use_ref = false;
        return TDM_OK;
    }
    const size_t HH = (size_t)c->p.H * c->p.H;
    std::vector<float> in(HH);
    if (is_device_ptr(intensity)) {
        TDM_CU(cudaMemcpy(in.data(), intensity, HH * sizeof(float), cudaMemcpyDeviceToHost));
    } else {
        std::memcpy(in.data(), intensity, HH * sizeof(float));
    }
    std::vector<float> inv(HH);
    for (size_t i = 0; i < HH; ++i) {
        const double v = in[i];
        if (!(v >= 0)) return fail(c, TDM_EINVAL, "tdm_set_reference_intensity: negative or NaN intensity");
        inv[i] = (float)(v != 0 ? 1.0 / std::sqrt(v) : 1.0);
    }
    if (!c->b.ref_inv && dev_alloc(c, &c->b.ref_inv, HH)) return fail(c, TDM_ENOMEM, "reference table allocation");
    TDM_CU(cudaMemcpy(c->b.ref_inv, inv.data(), HH * sizeof(float), cudaMemcpyHostToDevice));
    c->use_ref = true;
    return TDM_OK;
}

int tdm_synchronize(tdm_ctx* c) {
    if (!c) return TDM_EINVAL;
    TDM_CU(cudaStreamSynchronize(c->copy_stream));
    TDM_CU(cudaStreamSynchronize(c->vol_stream));
    TDM_CU(cudaStreamSynchronize(c->dl_stream));
    for (cudaStream_t l : c->lane_stream) TDM_CU(cudaStreamSynchronize(l));
    TDM_CU(cudaStreamSynchronize(c->stream));
    int err = 0;
    TDM_CU(cudaMemcpy(&err, c->b.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        cudaMemset(c->b.err, 0, sizeof(int));
        if (err & 2) return fail(c, TDM_ECUDA, "a bulk copy of hologram rows did not complete");
        if (err & 8) return fail(c, TDM_EDATA, "Herraez unwrapping: a 2 pi offset between merged groups beyond +-127");
        return fail(c, TDM_EDATA, "an Ewald-cap voxel fell outside the DIM_FINAL volume");
    }
    return TDM_OK;
}

void* tdm_stream(tdm_ctx* c) { return c ? (void*)c->stream : nullptr; }

int tdm_profile_count(void) { return K_COUNT; }

int tdm_profile(tdm_ctx* c, int enable) {
    if (!c) return TDM_EINVAL;
    TDM_CU(cudaStreamSynchronize(c->stream));
    prof_release(c);
    c->prof = enable != 0;
    return TDM_OK;
}

int tdm_profile_read(tdm_ctx* c, int index, const char** name, double* total_ms, int* launches) {
    if (!c || index < 0 || index >= K_COUNT) return TDM_EINVAL;
    TDM_CU(cudaStreamSynchronize(c->stream));
    TDM_CU(cudaStreamSynchronize(c->vol_stream));
    double t = 0;
    int n = 0;
    for (const ProfRec& r : c->prof_recs) {
        if (r.id != index) continue;
        float ms = 0;
        TDM_CU(cudaEventElapsedTime(&ms, r.a, r.b));
        t += ms;
        ++n;
    }
    if (name) *name = kKernelNames[index];
    if (total_ms) *total_ms = t;
    if (launches) *launches = n;
    return TDM_OK;
}
uint64_t tdm_launch_count(const tdm_ctx* c) { return c ? c->launches : 0; }

int tdm_cap_planes(const tdm_ctx* c, int* zmin, int* band) {
    if (!c) return TDM_EINVAL;
    if (zmin) *zmin = c->p.zmin;
    if (band) *band = c->p.band;
    return TDM_OK;
}

double tdm_stage_ms(const tdm_ctx* c, const char* stage) {
    if (!c || !stage) return -1;
    int a, b;
    if (!strcmp(stage, "extract")) a = 0, b = 1;
    else if (!strcmp(stage, "fields")) a = 1, b = 2;
    else if (!strcmp(stage, "map")) a = 2, b = 3;
    else if (!strcmp(stage, "gather")) a = 4, b = 5;
    else if (!strcmp(stage, "volume")) a = 4, b = 6;
    else if (!strcmp(stage, "total")) a = 0, b = 6;
    else return -1;
    float ms = -1;
    if (cudaEventElapsedTime(&ms, c->ev_stage[a], c->ev_stage[b]) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return ms;
}

// ---------------------------------------------------------------- stages
// Hologram staging for host stacks: a ring of slots of holo_chunk holograms
// (16-bit size) in the 2 chunk_cap holograms of b.holo_stage.
static int stage_slots(const tdm_ctx* c) {
    return std::max(1, std::min(kStageSlots, 2 * c->chunk_cap / c->holo_chunk));
}
static uint8_t* stage_slot(tdm_ctx* c, int s) {
    return c->b.holo_stage + (size_t)s * c->holo_chunk * c->p.H * c->p.H * 2;
}
// Chunks per hologram upload in the pipeline: up to 4 consecutive staging
// slots take one copy (a divisor of the ring's slot count, and at most a
// quarter of the ring, so later groups' uploads overlap the earlier ones'
// extraction).  With the volumes' downloads in flight, uploads of one
// 16-hologram chunk of 1024^2 (33 MB) kept the host link well below the rate
// it reaches in both directions at once with uploads of 126 MB or more;
// groups of 8 chunks did no better in the pipeline than groups of 4.
static int upload_group(int nslot) {
    for (int g = std::min(4, nslot / 4); g > 1; --g)
        if (nslot % g == 0) return g;
    return 1;
}

static int stage_extract(tdm_ctx* c, const void* holos, int bits, int n) {
    const Params& p = c->p;
    const size_t per = (size_t)p.H * p.H * (bits == 16 ? 2 : 1);
    if (is_device_ptr(holos)) return launch_extract(c, holos, bits, n, 0);
    // host holograms: chunked copies on the copy stream into a ring of staging slots
    const int nslot = stage_slots(c);
    for (int h0 = 0, k = 0; h0 < n; h0 += c->holo_chunk, ++k) {
        const int m = std::min(c->holo_chunk, n - h0);
        const int buf = k % nslot;
        uint8_t* dst = stage_slot(c, buf);
        TDM_CU(cudaStreamWaitEvent(c->copy_stream, c->ev_free[buf], 0));  // no-op before its first record
        TDM_CU(cudaMemcpyAsync(dst, static_cast<const char*>(holos) + h0 * per, m * per, cudaMemcpyHostToDevice,
                               c->copy_stream));
        TDM_CU(cudaEventRecord(c->ev_copy[buf], c->copy_stream));
        TDM_CU(cudaStreamWaitEvent(c->stream, c->ev_copy[buf], 0));
        if (int rc = launch_extract(c, dst, bits, m, h0)) return rc;
        TDM_CU(cudaEventRecord(c->ev_free[buf], c->stream));
    }
    return TDM_OK;
}

int tdm_extract(tdm_ctx* c, const void* holos, int bits, int n, float* spectra_out) {
    if (!c || !holos || (bits != 8 && bits != 16) || n <= 0 || n > c->max_angles)
        return fail(c, TDM_EINVAL, "tdm_extract: invalid argument");
    cudaSetDevice(c->device);
    TDM_CU(join_volume(c));
    TDM_CU(cudaEventRecord(c->ev_stage[0], c->stream));
    if (int rc = stage_extract(c, holos, bits, n)) return rc;
    TDM_CU(cudaEventRecord(c->ev_stage[1], c->stream));
    c->n_spectra = n;
    const size_t FF = (size_t)c->p.F * c->p.F;
    if (spectra_out)
        TDM_CU(cudaMemcpyAsync(spectra_out, c->b.spectra, n * FF * sizeof(float2), cudaMemcpyDefault, c->stream));
    if (!is_device_ptr(holos) || (spectra_out && !is_device_ptr(spectra_out))) return tdm_synchronize(c);
    return TDM_OK;
}

static int run_fields(tdm_ctx* c, const float* spectra_in, int n, float* fields_out, int32_t* posspec_out,
                      float* dph, float* dun, float* dam) {
    if (!c || n <= 0 || n > c->max_angles) return fail(c, TDM_EINVAL, "tdm_fields: invalid argument");
    cudaSetDevice(c->device);
    TDM_CU(join_volume(c));
    const size_t FF = (size_t)c->p.F * c->p.F;
    if (spectra_in && spectra_in != reinterpret_cast<float*>(c->b.spectra)) {
        TDM_CU(cudaMemcpyAsync(c->b.spectra, spectra_in, n * FF * sizeof(float2), cudaMemcpyDefault, c->stream));
    } else if (!spectra_in && n > c->n_spectra) {
        return fail(c, TDM_EINVAL, "tdm_fields: fewer spectra in the context than requested");
    }
    TDM_CU(cudaEventRecord(c->ev_stage[1], c->stream));
    if (int rc = launch_fields(c, 0, n, dph, dun, dam)) return fail(c, rc, "tdm_fields: kernel launch failed");
    TDM_CU(cudaEventRecord(c->ev_stage[2], c->stream));
    c->n_fields = n;
    bool host = (spectra_in && !is_device_ptr(spectra_in));
    if (fields_out) {
        TDM_CU(cudaMemcpyAsync(fields_out, c->b.fields, n * FF * sizeof(float2), cudaMemcpyDefault, c->stream));
        host |= !is_device_ptr(fields_out);
    }
    if (posspec_out) {
        if (is_device_ptr(posspec_out)) {
            Launch l(c, K_POSSPEC);
            k_unpack_posspec<<<(n + 255) / 256, 256, 0, c->stream>>>(c->b.posspec, n, posspec_out);
        } else {
            std::vector<int2> tmp(n);
            TDM_CU(cudaMemcpyAsync(tmp.data(), c->b.posspec, n * sizeof(int2), cudaMemcpyDeviceToHost, c->stream));
            TDM_CU(cudaStreamSynchronize(c->stream));
            for (int a = 0; a < n; ++a) {
                posspec_out[a] = tmp[a].x;
                posspec_out[n + a] = tmp[a].y;
            }
        }
    }
    if (host || dph || dun || dam) return tdm_synchronize(c);
    return TDM_OK;
}

int tdm_fields(tdm_ctx* c, const float* spectra_in, int n, float* fields_out, int32_t* posspec_out) {
    return run_fields(c, spectra_in, n, fields_out, posspec_out, nullptr, nullptr, nullptr);
}

int tdm_fields_debug(tdm_ctx* c, const float* spectra_in, int n, float* fields_out, int32_t* posspec_out,
                     float* phase_out, float* unwrapped_out, float* amp_out) {
    return run_fields(c, spectra_in, n, fields_out, posspec_out, phase_out, unwrapped_out, amp_out);
}

// Volume stage (and, with cap = true, the cap mapping of fields [0, n)
// first); outputs may be host or device memory.  Host outputs are written to
// device staging buffers and downloaded while the later passes run.
static int run_volume(tdm_ctx* c, int n, bool cap, float* re, float* im, uint8_t* otf, uint32_t* cnt,
                      bool wait = true, cudaStream_t st = nullptr, const CapRecs* rec = nullptr,
                      const int2* posspec = nullptr, cudaEvent_t ev_gathered = nullptr) {
    const Params& p = c->p;
    const size_t NT = (size_t)p.D * p.D * p.D;
    if (cap && launch_cap(c, 0, n)) return fail(c, TDM_ECUDA, "cap mapping launch failed");
    TDM_CU(cudaEventRecord(c->ev_stage[3], c->stream));
    Buffers& b = c->b;
    auto dev_or_stage = [&](auto* user, auto*& stage) -> decltype(user) {
        if (!user) return nullptr;
        if (is_device_ptr(user)) return user;
        if (!stage) {
            if (cudaMalloc(reinterpret_cast<void**>(&stage), NT * sizeof(*user)) != cudaSuccess) return nullptr;
        }
        return stage;
    };
    VolumeOut out;
    out.re = dev_or_stage(re, b.out_re);
    out.im = dev_or_stage(im, b.out_im);
    out.otf = dev_or_stage(otf, b.out_otf);
    out.cnt = dev_or_stage(cnt, b.out_cnt);
    if ((re && !out.re) || (im && !out.im) || (otf && !out.otf) || (cnt && !out.cnt))
        return fail(c, TDM_ENOMEM, "output staging allocation failed");
    if (re && out.re != re) out.host_re = re;
    if (im && out.im != im) out.host_im = im;
    if (otf && out.otf != otf) out.host_otf = otf;
    if (cnt && out.cnt != cnt) out.host_cnt = cnt;
    if (int rc = launch_volume(c, n, out, st ? st : c->stream, rec ? *rec : b.rec, posspec ? posspec : b.posspec,
                               ev_gathered))
        return fail(c, rc, "volume launch failed");
    const bool host = out.host_re || out.host_im || out.host_otf || out.host_cnt;
    return host && wait ? tdm_synchronize(c) : TDM_OK;
}

// Specular positions (x values then y values) into b.posspec.
static int set_posspec(tdm_ctx* c, const int32_t* posspec_in, int n, const char* who) {
    if (is_device_ptr(posspec_in)) {
        Launch l(c, K_POSSPEC);
        k_pack_posspec<<<(n + 255) / 256, 256, 0, c->stream>>>(posspec_in, n, c->b.posspec);
        return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
    }
    std::vector<int2> tmp(n);
    for (int a = 0; a < n; ++a) {
        if (posspec_in[a] < 0 || posspec_in[a] >= c->p.F || posspec_in[n + a] < 0 || posspec_in[n + a] >= c->p.F)
            return fail(c, TDM_EINVAL, std::string(who) + ": specular position outside the field");
        tmp[a] = make_int2(posspec_in[a], posspec_in[n + a]);
    }
    TDM_CU(cudaMemcpyAsync(c->b.posspec, tmp.data(), n * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
    TDM_CU(cudaStreamSynchronize(c->stream));
    return TDM_OK;
}

int tdm_reconstruct(tdm_ctx* c, const float* fields_in, const int32_t* posspec_in, int n, float* indice_out,
                    float* absorption_out, uint8_t* otf_out, uint32_t* counts_out) {
    if (!c || n <= 0 || n > c->max_angles) return fail(c, TDM_EINVAL, "tdm_reconstruct: invalid argument");
    cudaSetDevice(c->device);
    TDM_CU(join_volume(c));
    const size_t FF = (size_t)c->p.F * c->p.F;
    if ((!fields_in || !posspec_in) && n > c->n_fields)
        return fail(c, TDM_EINVAL, "tdm_reconstruct: fewer fields in the context than requested");
    if (fields_in && fields_in != reinterpret_cast<const float*>(c->b.fields))
        TDM_CU(cudaMemcpyAsync(c->b.fields, fields_in, n * FF * sizeof(float2), cudaMemcpyDefault, c->stream));
    if (posspec_in) {
        if (int rc = set_posspec(c, posspec_in, n, "tdm_reconstruct")) return rc;
        c->n_fields = std::max(c->n_fields, n);
    }
    TDM_CU(cudaEventRecord(c->ev_stage[2], c->stream));
    int rc = run_volume(c, n, true, indice_out, absorption_out, otf_out, counts_out);
    if (rc) return rc;
    c->n_caps = n;
    if (fields_in && !is_device_ptr(fields_in)) return tdm_synchronize(c);
    return TDM_OK;
}

// Scratch of the per-angle stages (the buffers sized chunk_cap angles) seen
// from chunk slot s on: the slots [s, s + chunk) of each.
struct ChunkScratch {
    float2* inter;
    float4* argpart;
    float2 *I1, *zph, *qc, *tq, *r1;
    float *phase, *amp, *gx, *unwrapped, *fit_part;
    double *beta, *phase_sum;
    unsigned* fit_done;
};

static ChunkScratch scratch_at(const tdm_ctx* c, int s) {
    const Buffers& b = c->b;
    const size_t FF = (size_t)c->p.F * c->p.F, LF = (size_t)c->p.L * c->p.F, S = (size_t)s;
    return ChunkScratch{b.inter + S * c->p.F * c->p.H, b.argpart + S * kArgPartsMax, b.I1 + S * FF, b.zph + S * FF,
                        b.qc + S * LF, b.tq + S * LF, b.r1 + S * FF, b.phase + S * FF, b.amp + S * FF,
                        b.gx + S * FF, b.unwrapped + S * FF, b.fit_part + S * 2 * 8 * kNC, b.beta + S * 2 * kNC,
                        b.phase_sum + S * kPhaseParts, b.fit_done + S * 2};
}

static void use_scratch(tdm_ctx* c, const ChunkScratch& k) {
    Buffers& b = c->b;
    b.inter = k.inter, b.argpart = k.argpart, b.I1 = k.I1, b.zph = k.zph, b.qc = k.qc, b.tq = k.tq, b.r1 = k.r1;
    b.phase = k.phase, b.amp = k.amp, b.gx = k.gx, b.unwrapped = k.unwrapped, b.fit_part = k.fit_part;
    b.beta = k.beta, b.phase_sum = k.phase_sum, b.fit_done = k.fit_done;
}

// Per-angle stages of the pipeline, streamed by hologram chunk: for each
// chunk, extraction, field formation and cap mapping run back to back (the
// chunk's spectra and fields stay in L2), and with host holograms the upload
// of later chunks overlaps them.  `lanes` consecutive chunks run at once (a
// per-chunk grid fills a fraction of the GPU): chunk k on lane k mod lanes,
// each lane a stream with its own chunk slots of the scratch buffers, forked
// from the context stream and joined back at the end.  The launchers read
// c->stream and the scratch pointers, which are switched per chunk here and
// restored on every return.
static int stage_angles(tdm_ctx* c, const void* holos, int bits, int n) {
    const Params& p = c->p;
    const size_t per = (size_t)p.H * p.H * (bits == 16 ? 2 : 1);
    const bool dev = is_device_ptr(holos);
    const int nchunks = (n + c->holo_chunk - 1) / c->holo_chunk;
    const int nl = std::max(1, std::min(std::min(c->lanes, kMaxLanes), std::min(c->chunk_cap / c->chunk, nchunks)));
    const int nslot = stage_slots(c), grp = upload_group(nslot);
    struct Restore {
        tdm_ctx* c;
        cudaStream_t main;
        ChunkScratch base;
        ~Restore() {
            c->stream = main;
            use_scratch(c, base);
        }
    } restore{c, c->stream, scratch_at(c, 0)};
    ChunkScratch lane_scratch[kMaxLanes];
    for (int l = 0; l < nl; ++l) lane_scratch[l] = scratch_at(c, l * c->chunk);
    if (nl > 1) {
        TDM_CU(cudaEventRecord(c->ev_lane_fork, restore.main));
        for (int l = 1; l < nl; ++l) TDM_CU(cudaStreamWaitEvent(c->lane_stream[l - 1], c->ev_lane_fork, 0));
    }
    for (int h0 = 0, k = 0; h0 < n; h0 += c->holo_chunk, ++k) {
        const int m = std::min(c->holo_chunk, n - h0);
        const int lane = k % nl;
        c->stream = lane ? c->lane_stream[lane - 1] : restore.main;
        use_scratch(c, lane_scratch[lane]);
        const void* src = static_cast<const char*>(holos) + h0 * per;
        const int buf = k % nslot, buf0 = buf - buf % grp;  // the chunk's slot and its group's first
        if (!dev) {
            // the upload that carries chunk k starts at chunk ks: a group's chunks
            // go up in one copy, except that the call's first chunk goes alone
            // (its extraction starts after one chunk, not a group)
            const int ks = k < grp ? std::min(k, 1) : k - k % grp;
            const size_t chunk_bytes = (size_t)c->holo_chunk * per;
            uint8_t* dst = stage_slot(c, buf0) + (size_t)(buf - buf0) * chunk_bytes;  // packed as on the host
            if (k == ks) {
                const int cnt = std::min(k == 0 && grp > 1 ? 1 : grp - (k % grp), nchunks - k);
                for (int q = 0; q < cnt; ++q)
                    TDM_CU(cudaStreamWaitEvent(c->copy_stream, c->ev_free[buf + q], 0));  // no-op before a first record
                const size_t bytes = (size_t)std::min(cnt * c->holo_chunk, n - h0) * per;
                TDM_CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->copy_stream));
                TDM_CU(cudaEventRecord(c->ev_copy[buf], c->copy_stream));
            }
            TDM_CU(cudaStreamWaitEvent(c->stream, c->ev_copy[ks % nslot], 0));
            src = dst;
        }
        // the extraction leaves the specular search's partial winners for the
        // field stage; with C_ABER the cap row pass forms the fields
        const int parts = launch_extract(c, src, bits, m, h0, true);
        if (parts <= 0) return fail(c, parts ? parts : TDM_ECUDA, "extraction launch failed");
        if (!dev) TDM_CU(cudaEventRecord(c->ev_free[buf], c->stream));
        const bool form_in_cap = p.c_aber != 0;
        if (int rc = launch_fields(c, h0, m, nullptr, nullptr, nullptr, parts, !form_in_cap))
            return fail(c, rc, "fields launch failed");
        if (int rc = launch_cap(c, h0, m, form_in_cap)) return fail(c, rc, "cap mapping launch failed");
    }
    for (int l = 1; l < nl; ++l) {
        TDM_CU(cudaEventRecord(c->ev_lane_join[l - 1], c->lane_stream[l - 1]));
        TDM_CU(cudaStreamWaitEvent(restore.main, c->ev_lane_join[l - 1], 0));
    }
    return TDM_OK;
}

static int pipeline(tdm_ctx* c, const void* holos, int bits, int n, float* indice_out, float* absorption_out,
                    uint8_t* otf_out, uint32_t* counts_out, int32_t* posspec_out, bool wait) {
    if (!c || !holos || (bits != 8 && bits != 16) || n <= 0 || n > c->max_angles)
        return fail(c, TDM_EINVAL, "tdm_pipeline: invalid argument");
    cudaSetDevice(c->device);
    // The per-angle stages run on c->stream, the volume stage on vol_stream, so
    // that this call's volume stage overlaps the next call's per-angle stages.
    // This call's cap records go to rec_buf[par], after the gather of two calls
    // ago has read it; the specular positions its gather reads are copied aside.
    const int par = c->rec_parity;
    c->b.rec = c->b.rec_buf[par];
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    TDM_CU(cudaStreamIsCapturing(c->stream, &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    if (!capturing) TDM_CU(cudaStreamWaitEvent(c->stream, c->ev_rec_free[par], 0));  // a graph is ordered by its launches
    TDM_CU(cudaEventRecord(c->ev_stage[0], c->stream));
    if (int rc = stage_angles(c, holos, bits, n)) return rc;
    TDM_CU(cudaEventRecord(c->ev_stage[1], c->stream));  // extract, fields and map are interleaved
    TDM_CU(cudaEventRecord(c->ev_stage[2], c->stream));
    c->n_spectra = n;
    c->n_fields = n;
    c->n_caps = n;
    if (posspec_out && is_device_ptr(posspec_out)) {
        Launch l(c, K_POSSPEC);
        k_unpack_posspec<<<(n + 255) / 256, 256, 0, c->stream>>>(c->b.posspec, n, posspec_out);
    }
    TDM_CU(cudaMemcpyAsync(c->b.posspec_vol[par], c->b.posspec, n * sizeof(int2), cudaMemcpyDeviceToDevice,
                           c->stream));
    TDM_CU(cudaEventRecord(c->ev_angles, c->stream));
    TDM_CU(cudaStreamWaitEvent(c->vol_stream, c->ev_angles, 0));
    int rc = run_volume(c, n, false, indice_out, absorption_out, otf_out, counts_out, wait, c->vol_stream,
                        &c->b.rec_buf[par], c->b.posspec_vol[par], c->ev_rec_free[par]);
    if (rc) return rc;
    TDM_CU(cudaEventRecord(c->ev_vol_last, c->vol_stream));
    c->rec_parity ^= 1;
    if (capturing) TDM_CU(join_volume(c));  // a capture must end joined
    if (posspec_out && !is_device_ptr(posspec_out)) {
        std::vector<int2> tmp(n);
        TDM_CU(cudaMemcpyAsync(tmp.data(), c->b.posspec, n * sizeof(int2), cudaMemcpyDeviceToHost, c->stream));
        TDM_CU(cudaStreamSynchronize(c->stream));
        for (int a = 0; a < n; ++a) {
            posspec_out[a] = tmp[a].x;
            posspec_out[n + a] = tmp[a].y;
        }
    }
    if (wait && !is_device_ptr(holos)) return tdm_synchronize(c);
    return TDM_OK;
}

int tdm_pipeline(tdm_ctx* c, const void* holos, int bits, int n, float* indice_out, float* absorption_out,
                 uint8_t* otf_out, uint32_t* counts_out, int32_t* posspec_out) {
    return pipeline(c, holos, bits, n, indice_out, absorption_out, otf_out, counts_out, posspec_out, true);
}

int tdm_pipeline_async(tdm_ctx* c, const void* holos, int bits, int n, float* indice_out, float* absorption_out,
                       uint8_t* otf_out, uint32_t* counts_out) {
    return pipeline(c, holos, bits, n, indice_out, absorption_out, otf_out, counts_out, nullptr, false);
}

// ---------------------------------------------------------------- forward operator, adjoint, regularised reconstruction
static int ensure_operator_buffers(tdm_ctx* c) {
    const size_t NT = (size_t)c->p.D * c->p.D * c->p.D, MF = (size_t)c->max_angles * c->p.F * c->p.F;
    for (auto& v : c->b.xv)
        if (!v && dev_alloc(c, &v, NT)) return TDM_ENOMEM;
    if (!c->b.caps && dev_alloc(c, &c->b.caps, MF)) return TDM_ENOMEM;
    if (!c->b.rec2.val && (dev_alloc(c, &c->b.rec2.val, MF) || dev_alloc(c, &c->b.rec2.z, MF))) return TDM_ENOMEM;
    if (!c->b.misfit && dev_alloc(c, &c->b.misfit, 1)) return TDM_ENOMEM;
    return TDM_OK;
}

static int operator_setup(tdm_ctx* c, int n, const int32_t* posspec, const char* who) {
    if (!c || n <= 0 || n > c->max_angles) return fail(c, TDM_EINVAL, std::string(who) + ": invalid argument");
    cudaSetDevice(c->device);
    TDM_CU(join_volume(c));
    if (posspec) {
        if (int rc = set_posspec(c, posspec, n, who)) return rc;
        c->n_fields = std::max(c->n_fields, n);
    } else if (n > c->n_fields) {
        return fail(c, TDM_EINVAL, std::string(who) + ": no specular positions for that many angles in the context");
    }
    if (ensure_operator_buffers(c)) return fail(c, TDM_ENOMEM, std::string(who) + ": buffer allocation failed");
    return TDM_OK;
}

int tdm_forward(tdm_ctx* c, const float* index, const float* absorption, int n, const int32_t* posspec,
                float* caps_out) {
    if (!index || !caps_out) return fail(c, TDM_EINVAL, "tdm_forward: invalid argument");
    if (int rc = operator_setup(c, n, posspec, "tdm_forward")) return rc;
    const size_t NT = (size_t)c->p.D * c->p.D * c->p.D, FF = (size_t)c->p.F * c->p.F;
    const float* xn = index;
    const float* xk = absorption;
    if (!is_device_ptr(xn)) {
        TDM_CU(cudaMemcpyAsync(c->b.xv[0], xn, NT * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        xn = c->b.xv[0];
    }
    if (xk && !is_device_ptr(xk)) {
        TDM_CU(cudaMemcpyAsync(c->b.xv[1], xk, NT * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        xk = c->b.xv[1];
    }
    const bool host_out = !is_device_ptr(caps_out);
    float2* caps = host_out ? c->b.caps : reinterpret_cast<float2*>(caps_out);
    if (int rc = launch_forward(c, xn, xk, n, caps, nullptr, CapRecs{}, nullptr))
        return fail(c, rc, "tdm_forward: launch failed");
    if (host_out)
        TDM_CU(cudaMemcpyAsync(caps_out, caps, n * FF * sizeof(float2), cudaMemcpyDeviceToHost, c->stream));
    const bool host = host_out || !is_device_ptr(index) || (absorption && !is_device_ptr(absorption));
    return host ? tdm_synchronize(c) : TDM_OK;
}

int tdm_adjoint(tdm_ctx* c, const float* caps, int n, const int32_t* posspec, float* index_out,
                float* absorption_out) {
    if (!caps || !index_out) return fail(c, TDM_EINVAL, "tdm_adjoint: invalid argument");
    if (int rc = operator_setup(c, n, posspec, "tdm_adjoint")) return rc;
    const size_t NT = (size_t)c->p.D * c->p.D * c->p.D, FF = (size_t)c->p.F * c->p.F;
    const float2* cv = reinterpret_cast<const float2*>(caps);
    if (!is_device_ptr(caps)) {
        TDM_CU(cudaMemcpyAsync(c->b.caps, caps, n * FF * sizeof(float2), cudaMemcpyHostToDevice, c->stream));
        cv = c->b.caps;
    }
    float* xn = is_device_ptr(index_out) ? index_out : c->b.xv[4];
    float* xk = absorption_out ? (is_device_ptr(absorption_out) ? absorption_out : c->b.xv[5]) : nullptr;
    if (int rc = launch_cap_pack(c, cv, n, c->b.rec2)) return fail(c, rc, "tdm_adjoint: launch failed");
    if (int rc = launch_adjoint(c, c->b.rec2, n, xn, xk, false)) return fail(c, rc, "tdm_adjoint: launch failed");
    bool host = !is_device_ptr(caps);
    if (xn != index_out) {
        TDM_CU(cudaMemcpyAsync(index_out, xn, NT * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
        host = true;
    }
    if (xk && xk != absorption_out) {
        TDM_CU(cudaMemcpyAsync(absorption_out, xk, NT * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
        host = true;
    }
    return host ? tdm_synchronize(c) : TDM_OK;
}

int tdm_tv_reconstruct(tdm_ctx* c, const float* caps, int n, const int32_t* posspec, const tdm_tv_opts* o,
                       float* index_io, float* absorption_io, tdm_tv_report* report) {
    if (!o || !index_io || o->iterations < 0) return fail(c, TDM_EINVAL, "tdm_tv_reconstruct: invalid argument");
    if (int rc = operator_setup(c, n, posspec, "tdm_tv_reconstruct")) return rc;
    Buffers& b = c->b;
    const size_t NT = (size_t)c->p.D * c->p.D * c->p.D, FF = (size_t)c->p.F * c->p.F;
    if (caps) {  // the data: cap records of the given cap values
        const float2* cv = reinterpret_cast<const float2*>(caps);
        if (!is_device_ptr(caps)) {
            TDM_CU(cudaMemcpyAsync(b.caps, caps, n * FF * sizeof(float2), cudaMemcpyHostToDevice, c->stream));
            cv = b.caps;
        }
        if (int rc = launch_cap_pack(c, cv, n, b.rec)) return fail(c, rc, "tdm_tv_reconstruct: launch failed");
        c->n_caps = n;
    } else if (n > c->n_caps) {
        return fail(c, TDM_EINVAL, "tdm_tv_reconstruct: no cap records for that many angles in the context");
    }
    const bool absn = absorption_io != nullptr;
    float* xn = b.xv[0];
    float* xk = absn ? b.xv[1] : nullptr;
    float* xn2 = b.xv[2];
    float* xk2 = absn ? b.xv[3] : nullptr;
    float* gn = b.xv[4];
    float* gk = absn ? b.xv[5] : nullptr;
    if (o->init == 1) {
        if (int rc = launch_adjoint(c, b.rec, n, xn, xk, true)) return fail(c, rc, "tdm_tv_reconstruct: launch failed");
    } else {
        TDM_CU(cudaMemcpyAsync(xn, index_io, NT * sizeof(float), cudaMemcpyDefault, c->stream));
        if (absn) TDM_CU(cudaMemcpyAsync(xk, absorption_io, NT * sizeof(float), cudaMemcpyDefault, c->stream));
    }
    // TV steps relative to each channel's box range (absolute when unbounded)
    auto range = [](float lo, float hi) { return std::isfinite(hi - lo) && hi > lo ? hi - lo : 1.0f; };
    const float tv_n = o->tv_weight * range(o->index_min, o->index_max);
    const float tv_k = o->tv_weight * range(o->absorption_min, o->absorption_max);
    cudaEvent_t t0 = prof_event(c), t1 = prof_event(c);
    TDM_CU(cudaEventRecord(t0, c->stream));
    double first = -1, last = -1;
    for (int it = 0; it < o->iterations; ++it) {
        TDM_CU(cudaMemsetAsync(b.misfit, 0, sizeof(double), c->stream));
        if (int rc = launch_forward(c, xn, xk, n, nullptr, b.rec.val, b.rec2, b.misfit))
            return fail(c, rc, "tdm_tv_reconstruct: launch failed");
        if (it == 0 || it == o->iterations - 1) {
            double m = 0;
            TDM_CU(cudaMemcpyAsync(&m, b.misfit, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
            TDM_CU(cudaStreamSynchronize(c->stream));
            (it == 0 ? first : last) = m;
            if (o->iterations == 1) last = m;
        }
        if (int rc = launch_adjoint(c, b.rec2, n, gn, gk, true)) return fail(c, rc, "tdm_tv_reconstruct: launch failed");
        if (int rc = launch_tv_step(c, xn, xk, gn, gk, o->step, tv_n, tv_k, o->tv_eps, o->index_min, o->index_max,
                                    o->absorption_min, o->absorption_max, xn2, xk2))
            return fail(c, rc, "tdm_tv_reconstruct: launch failed");
        std::swap(xn, xn2);
        std::swap(xk, xk2);
    }
    TDM_CU(cudaEventRecord(t1, c->stream));
    TDM_CU(cudaMemcpyAsync(index_io, xn, NT * sizeof(float), cudaMemcpyDefault, c->stream));
    if (absn) TDM_CU(cudaMemcpyAsync(absorption_io, xk, NT * sizeof(float), cudaMemcpyDefault, c->stream));
    if (int rc = tdm_synchronize(c)) return rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    c->ev_pool.push_back(t0);
    c->ev_pool.push_back(t1);
    if (report) {
        report->iterations = o->iterations;
        report->misfit_first = first;
        report->misfit_last = last;
        report->seconds = ms / 1e3;
    }
    return TDM_OK;
}

// ---------------------------------------------------------------- batched acquisitions
struct tdm_batch {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

int tdm_batch_create(int count, tdm_ctx* const* ctxs, const void* const* holos, const int* bits, const int* n,
                     float* const* indice, float* const* absorption, uint8_t* const* otf, tdm_batch** out) {
    if (!out || count <= 0 || !ctxs || !holos || !bits || !n) return TDM_EINVAL;
    *out = nullptr;
    for (int i = 0; i < count; ++i) {
        if (!ctxs[i] || !holos[i] || !is_device_ptr(holos[i])) return TDM_EINVAL;
        const void* outs[3] = {indice ? indice[i] : nullptr, absorption ? absorption[i] : nullptr,
                               otf ? otf[i] : nullptr};
        for (const void* o : outs)
            if (o && !is_device_ptr(o)) return fail(ctxs[i], TDM_EINVAL, "tdm_batch_create: outputs must be device memory");
    }
    auto* b = new tdm_batch;
    if (cudaGraphCreate(&b->graph, 0) != cudaSuccess) {
        delete b;
        return TDM_ECUDA;
    }
    for (int i = 0; i < count; ++i) {
        tdm_ctx* c = ctxs[i];
        cudaSetDevice(c->device);
        // relaxed: the pipeline sets kernel attributes while it is captured
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
            tdm_batch_destroy(b);
            return cuda_fail(c, cudaGetLastError(), "tdm_batch_create: capture");
        }
        const int rc = pipeline(c, holos[i], bits[i], n[i], indice ? indice[i] : nullptr,
                                absorption ? absorption[i] : nullptr, otf ? otf[i] : nullptr, nullptr, nullptr, false);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        cudaGraphNode_t node;
        if (rc || e != cudaSuccess || cudaGraphAddChildGraphNode(&node, b->graph, nullptr, 0, g) != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            tdm_batch_destroy(b);
            return rc ? rc : cuda_fail(c, e ? e : cudaGetLastError(), "tdm_batch_create: graph");
        }
        cudaGraphDestroy(g);  // the child node holds a copy
    }
    if (cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess) {
        tdm_batch_destroy(b);
        return cuda_fail(ctxs[0], cudaGetLastError(), "tdm_batch_create: instantiate");
    }
    *out = b;
    return TDM_OK;
}

int tdm_batch_launch(tdm_batch* b, void* stream) {
    if (!b || !b->exec) return TDM_EINVAL;
    return cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)) == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

int tdm_batch_destroy(tdm_batch* b) {
    if (!b) return TDM_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    delete b;
    return TDM_OK;
}

// ---------------------------------------------------------------- autotuning
int tdm_set_wait_limit(tdm_ctx* c, long long polls) {
    if (!c || polls > (long long)kMbarPolls) return fail(c, TDM_EINVAL, "tdm_set_wait_limit: at most 2^24 polls");
    cudaSetDevice(c->device);
    if (int rc = tdm_synchronize(c)) return rc;  // queued extractions keep the bound they were launched with
    c->wait_polls = polls < 0 ? kMbarPolls : (uint32_t)polls;
    return TDM_OK;
}

int tdm_set_schedule(tdm_ctx* c, int chunk, int lanes) {
    if (!c || chunk < 1 || lanes < 1 || lanes > kMaxLanes || chunk * lanes > c->chunk_cap)
        return fail(c, TDM_EINVAL, "tdm_set_schedule: need 1 <= lanes <= 8 and chunk * lanes <= the chunk capacity");
    cudaSetDevice(c->device);
    if (int rc = tdm_synchronize(c)) return rc;  // the staging ring's slots move with the chunk size
    c->chunk = c->holo_chunk = chunk;
    c->lanes = lanes;
    return TDM_OK;
}

int tdm_autotune(tdm_ctx* c, const void* holos, int bits, int n, int* chunk_out) {
    if (!c || !holos || !is_device_ptr(holos) || (bits != 8 && bits != 16) || n <= 0 || n > c->max_angles)
        return fail(c, TDM_EINVAL, "tdm_autotune: invalid argument (device holograms required)");
    cudaSetDevice(c->device);
    if (int rc = tdm_synchronize(c)) return rc;
    const int cands[][2] = {{16, 4}, {16, 2}, {8, 4}, {12, 4}, {32, 2}, {16, 6}, {32, 4}};
    int best = c->chunk, best_lanes = c->lanes;
    float best_ms = 0;
    cudaEvent_t t0 = prof_event(c), t1 = prof_event(c);
    int rc = TDM_OK;
    for (const auto& cand : cands) {
        if (cand[0] * cand[1] > c->chunk_cap) continue;
        c->chunk = c->holo_chunk = cand[0];
        c->lanes = cand[1];
        rc = pipeline(c, holos, bits, n, nullptr, nullptr, nullptr, nullptr, nullptr, false);  // warm-up
        if (!rc && cudaEventRecord(t0, c->stream) != cudaSuccess) rc = TDM_ECUDA;
        for (int r = 0; r < 2 && !rc; ++r) rc = pipeline(c, holos, bits, n, nullptr, nullptr, nullptr, nullptr, nullptr, false);
        if (!rc && (join_volume(c) != cudaSuccess || cudaEventRecord(t1, c->stream) != cudaSuccess)) rc = TDM_ECUDA;
        if (!rc) rc = tdm_synchronize(c);
        float ms = 0;
        if (!rc && cudaEventElapsedTime(&ms, t0, t1) != cudaSuccess) rc = TDM_ECUDA;
        if (rc) break;
        if (best_ms == 0 || ms < best_ms) {
            best_ms = ms;
            best = cand[0];
            best_lanes = cand[1];
        }
    }
    c->ev_pool.push_back(t0);
    c->ev_pool.push_back(t1);
    c->chunk = c->holo_chunk = best;
    c->lanes = best_lanes;
    if (rc) return rc;
    if (chunk_out) *chunk_out = best;
    return TDM_OK;
}

}  // extern "C"
