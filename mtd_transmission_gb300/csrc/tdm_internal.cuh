// Internal declarations shared by the kernel and API translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tdm.h"
#include "fft_core.cuh"
#include "argmax.cuh"

namespace tdm {

constexpr int kNC = 15;  // degree-4 2D polynomial: 15 monomials
constexpr int kOutSlabs = 8;  // x-pass slabs whose outputs are downloaded while the next slab runs
constexpr int kOutEvents = kOutSlabs + 2;
constexpr int kMaxLanes = 8;    // chunks of the per-angle stages in flight at once
constexpr int kStageSlots = 16; // hologram upload slots of one chunk each
constexpr int kChunkCapMax = 128;  // angles of per-chunk scratch (all lanes together), at most

// Cap records of a stack: per angle and FFT bin ([angle][ky][kx]) the cap
// value (the cell's contribution, 0 outside the cap cells) and the cell's
// volume plane (-1 outside the cells).
struct CapRecs {
    float2* val = nullptr;
    int16_t* z = nullptr;
};

// Device-side parameters of one volume, fixed at context creation.
struct Params {
    int H, N, F, L, D;
    int x0, y0;              // crop corner in the fftshifted hologram spectrum
    int born, c_aber, deroul;
    int volkov;              // VOLKOV: 1 Volkov unwrapping, 0 Herraez
    int disc_thr;            // fd^2 < disc_thr  <=>  fd^2 < COEF_NA_OBJ_LIMIT * N^2
    int zmin, band;          // cap planes z in [zmin, zmin + band)
    int r2i;                 // rayon^2 when below 2^24 (cap heights as float sqrt of exact integers), else 0
    double rayon, inv_rayon;
    float cap_scale;         // (k0/pi)*(-2pi) of retroPropag_Born, k0 in float
    float dx2;               // tailleTheoPixelUborn^2
    float out_scale;         // Delta_f^3 * (-1/(2 n0 kv^2))
};

// Device buffers (all owned by the context).
// Per-CTA sums of an angle's wrapped phase kept for the Volkov unwrap's mean
// term (one per CTA of the field column pass).
constexpr int kPhaseParts = 64;

struct Buffers {
    float2* tw = nullptr;          // kTwTotal twiddles (twiddle_table)
    float2* win_h = nullptr;       // H, hologram window with sign (hologram_window)
    float* ref_inv = nullptr;      // H*H, 1 / reference amplitude (tdm_set_reference_intensity), on first use
    float* tuk_f = nullptr;        // F, field Tukey alpha 0.1 (1D factor)
    double* s_tab = nullptr;       // F*F, sqrt(rayon^2 - fd^2) at [fdy+N][fdx+N]
    float* s_tabf = nullptr;       // float copy
    float2* wq = nullptr;          // 4F, exp(-2 pi i k / 4F): twiddles of the mixed-radix passes
    uint8_t* holo_stage = nullptr; // host staging: 2 x chunk x H*H*2 bytes
    float2* inter = nullptr;       // chunk x F x H (extraction row pass, kx band column-major)
    float2* spectra = nullptr;     // max_angles x F*F
    int2* posspec = nullptr;       // max_angles
    float2* specval = nullptr;     // max_angles
    float4* argpart = nullptr;     // chunk x kArgPartsMax partial winners of the specular search
    float2* I1 = nullptr;          // chunk x F*F
    float* phase = nullptr;        // chunk x F*F
    float* amp = nullptr;          // chunk x F*F
    float2* zph = nullptr;         // chunk x F*F unit phasor exp(i phase) (Volkov input)
    float* gx = nullptr;           // chunk x F*F (right half of the mirror's gx, per image row)
    float2* qc = nullptr;          // chunk x L*F: Volkov, F*F per angle: per column the DCT-II of gx and DST-II of gy;
                                   // Herraez, sort scratch
    float2* tq = nullptr;          // chunk x L*F: Volkov, F*F floats per angle: the Poisson solve's rows;
                                   // Herraez, sort scratch
    double* phase_sum = nullptr;   // chunk x kPhaseParts: the field column pass's per-CTA sums of the wrapped phase
    float* unwrapped = nullptr;    // chunk x F*F
    int* hz_rand = nullptr;        // VOLKOV 0: max_angles x (4F - 4) border rand() draws (crand_border_table)
    double* beta = nullptr;        // chunk x 2 x kNC
    float* fit_part = nullptr;     // chunk x 2 x 8 x kNC slice sums of the fits
    unsigned* fit_done = nullptr;  // chunk x 2 finished-slice counters (zero between launches)
    float2* fields = nullptr;      // max_angles x F*F
    float2* r1 = nullptr;          // chunk x F*F
    CapRecs rec;                   // max_angles x F*F cap records: rec_buf[i]
    CapRecs rec_buf[2];            // the two cap-record buffers of consecutive pipeline calls
    int2* posspec_vol[2] = {};     // max_angles: specular positions read by the volume stage of those calls
    float2* vol = nullptr;         // D^3 complex, [y][x][z] layout
    float* out_re = nullptr;       // D^3 staging when the caller's output is in host memory
    float* out_im = nullptr;
    uint8_t* out_otf = nullptr;
    uint32_t* out_cnt = nullptr;
    int* samp_idx = nullptr;       // nsamp aberration sample pixels
    float* samp_q = nullptr;       // nsamp x kNC orthonormal basis values
    double* rinv = nullptr;        // kNC x kNC: monomial coefficients from basis coefficients
    int* err = nullptr;            // device error flags
    // forward operator / adjoint / regularised reconstruction (allocated on first use)
    float* xv[6] = {};             // D^3 each: iterate index/absorption (x2, double buffered), gradient index/absorption
    float2* caps = nullptr;        // max_angles x F*F cap values staged for host callers
    CapRecs rec2;                  // max_angles x F*F residual / adjoint-input cap records
    double* misfit = nullptr;      // data misfit accumulator
};

// Kernel names for the opt-in per-launch profiler (tdm_profile).
enum KernelId {
    K_EXTRACT_ROWS, K_EXTRACT_COLS, K_ARGMAX, K_FIELD_ROWS, K_FIELD_COLS, K_VOLKOV_ROWS, K_VOLKOV_COLS,
    K_VOLKOV_INTEG_ROWS, K_VOLKOV_INTEG_COLS, K_ABER_FIT, K_FORM, K_CAP_ROWS, K_CAP_COLS, K_GATHER,
    K_YPASS, K_XPASS, K_POSSPEC, K_ZPASS, K_HERRAEZ, K_COUNT
};
extern const char* const kKernelNames[K_COUNT];

struct ProfRec {
    int id;
    cudaEvent_t a, b;
};

}  // namespace tdm

struct tdm_ctx {
    tdm_geom g{};
    tdm_derived dv{};
    tdm::Params p{};
    tdm::Buffers b{};
    int max_angles = 0;
    int chunk = 16;              // angles per chunk of the per-angle stages (tdm_set_schedule, tdm_autotune)
    int holo_chunk = 16;         // holograms per extraction chunk (equal to chunk)
    int lanes = 4;               // chunks in flight at once; lanes * chunk <= chunk_cap
    int chunk_cap = 64;          // angles of per-chunk scratch: min(128, max_angles rounded up to 16)
    int nsamp = 0;
    int device = 0;
    int2 tuk_h_flat{0, -1}, tuk_f_flat{0, -1};  // where the hologram / field windows are exactly 1
    uint32_t wait_polls = 1u << 24;  // polls of a bulk copy's first wait in the extraction (tdm_set_wait_limit)
    bool use_ref = false;        // holograms divided by the reference amplitude (b.ref_inv)
    int n_fields = 0;            // angles held in b.fields / b.posspec
    int n_spectra = 0;           // angles held in b.spectra
    int n_caps = 0;              // angles held in b.rec (cap records)
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // hologram uploads
    cudaStream_t dl_stream = nullptr;    // output downloads (a second copy engine)
    // downloads of the staged outputs done, per part (x-pass slabs, then counts, then OTF): a volume
    // stage waits for the previous volume's download of a part just before it rewrites that part
    cudaEvent_t ev_dl[tdm::kOutEvents] = {};
    // tdm_pipeline runs each volume's stage (gather, z/y/x passes) on vol_stream, so that it
    // overlaps the next call's per-angle stages; the cap records and the specular positions the
    // volume stage reads are double buffered
    cudaStream_t vol_stream = nullptr;
    // the per-angle stages run `lanes` chunks at once: chunk k on lane k mod lanes (lane 0 is
    // `stream`, lane l > 0 is lane_stream[l - 1]) with chunk slots [l chunk, (l + 1) chunk) of the
    // scratch buffers
    cudaStream_t lane_stream[tdm::kMaxLanes - 1] = {};
    cudaEvent_t ev_lane_fork = nullptr;
    cudaEvent_t ev_lane_join[tdm::kMaxLanes - 1] = {};
    cudaEvent_t ev_angles = nullptr;     // per-angle stages of the current call done (stream)
    cudaEvent_t ev_vol_last = nullptr;   // last volume stage queued on vol_stream
    cudaEvent_t ev_rec_free[2] = {};     // gather that read rec_buf[i] done
    int rec_parity = 0;
    cudaEvent_t ev_copy[tdm::kStageSlots] = {};  // upload into hologram staging slot s done
    cudaEvent_t ev_free[tdm::kStageSlots] = {};  // extraction that read slot s done
    cudaEvent_t ev_stage[8] = {};
    cudaEvent_t ev_out[tdm::kOutEvents] = {};  // downloads of the volume outputs (copy stream)
    uint64_t launches = 0;
    bool prof = false;
    std::vector<tdm::ProfRec> prof_recs;
    std::vector<cudaEvent_t> ev_pool;
    std::string last_error;
};

// Kernel launchers (defined in the kernel translation units).
namespace tdm {
// Dynamic shared memory of the cap gather for a cap band of `band` planes and
// n angles (the CTA keeps its list of angles in shared memory).
size_t gather_smem_bytes(int D, int band, int n);
constexpr size_t kMaxSmemPerCta = 227 * 1024;
// Scope around one kernel launch on c->stream: counts the launch and, when
// profiling is on, brackets it with a pair of CUDA events.
cudaEvent_t prof_event(tdm_ctx* c);
struct Launch {
    tdm_ctx* c;
    int id;
    cudaStream_t st;
    cudaEvent_t b = nullptr;
    Launch(tdm_ctx* ctx, int kid, cudaStream_t stream = nullptr) : c(ctx), id(kid), st(stream ? stream : ctx->stream) {
        if (c->prof) {
            cudaEvent_t a = prof_event(c);
            b = prof_event(c);
            cudaEventRecord(a, st);
            c->prof_recs.push_back(ProfRec{id, a, b});
        }
    }
    ~Launch() {
        if (b) cudaEventRecord(b, st);
        c->launches++;
    }
};
// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) of kernel fn on the current
// device, made once per kernel, device and size (the launchers run per chunk,
// and the attribute call costs host time on each).  It is set for any size:
// a kernel's static shared memory counts against the default 48 KB too.  The
// attribute belongs to the function, shared by every context on the device,
// so it is only ever raised: a context of another geometry asking for less
// must not lower it under a launch (or a captured graph) that needs more.
cudaError_t max_dynamic_smem(const void* fn, size_t bytes);

// Extraction of holograms [0, n) from device memory into spectra[a0, a0 + n).
// With argmax = true (n at most one chunk), the column pass also leaves the
// specular search's partial winners of each angle in b.argpart; the return
// value is then the number of partial records per angle (> 0).
int launch_extract(tdm_ctx* c, const void* holos_dev, int bits, int n, int a0, bool argmax = false);
// Per-angle field formation for spectra [a0, a0 + n).  argparts > 0: the
// extraction left that many partial winners per angle (one chunk only);
// form = false (C_ABER pipeline): the fields are formed by the cap row pass.
// Herraez unwrapping (VOLKOV 0) of the chunk's m wrapped phases (b.phase ->
// b.unwrapped), stack angles a0 .. a0 + m - 1; F <= 256.
int launch_herraez(tdm_ctx* c, int a0, int m);
size_t herraez_gather_smem(int F);
int launch_fields(tdm_ctx* c, int a0, int n, float* dbg_phase, float* dbg_unwrapped, float* dbg_amp,
                  int argparts = 0, bool form = true);
// Per-field spectra and cap contributions for fields [a0, a0 + n); with
// form = true (one chunk, after launch_fields(..., form = false)) the fields
// are formed from the chunk's unwrapped phase, amplitude and fits on the fly
// (and stored in b.fields).
int launch_cap(tdm_ctx* c, int a0, int n, bool form = false);
// The same two stages for field sizes that are not powers of two (the
// mixed-radix engine, fft_generic.cuh; k_generic.cu).
int launch_fields_generic(tdm_ctx* c, int a0, int n, float* dbg_phase, float* dbg_unwrapped, float* dbg_amp,
                          int argparts, bool form);
int launch_cap_generic(tdm_ctx* c, int a0, int n, bool form);
// Field sizes the mixed-radix passes are compiled for (2 NXMAX, not powers of two).
bool generic_field_size(int F);
// Pieces of the field stage shared by both engines (k_fields.cu): the
// standalone specular-search partials of m spectra (returns the records per
// angle), the aberration fits and the field formation of the chunk's m angles.
int launch_argmax_part(tdm_ctx* c, const float2* spec, int m);
void launch_aber_fit(tdm_ctx* c, const float* unw, int m);
void launch_form(tdm_ctx* c, const float* unw, int g0, int m);
// Outputs of the volume stage: the device buffers the kernels write and, for
// each caller buffer in host memory, the host destination its device copy is
// downloaded to on the copy stream as soon as the pass that completes it has
// run (the index and absorption volumes slab by slab during the x pass).
struct VolumeOut {
    float* re = nullptr;
    float* im = nullptr;
    uint8_t* otf = nullptr;
    uint32_t* cnt = nullptr;
    float* host_re = nullptr;
    float* host_im = nullptr;
    uint8_t* host_otf = nullptr;
    uint32_t* host_cnt = nullptr;
};
// Forward operator of the cap mapping on the D^3 volumes xn + i xk ([z][y][x];
// xk may be null): caps (n x F^2, may be null) = the spectrum at each angle's
// cap cells; with data (cap records), res = spectrum - data on the data's
// cells and *misfit += sum |res|^2.  Uses b.vol.
int launch_forward(tdm_ctx* c, const float* xn, const float* xk, int n, float2* caps, const float2* data,
                   CapRecs res, double* misfit);
// Adjoint of the forward operator applied to cap records (unnormalised
// scatter, z/y/x passes); with normalize, the hit-count-normalised scatter and
// the reconstruction's own scale (the single-pass reconstruction of recs).
int launch_adjoint(tdm_ctx* c, CapRecs recs, int n, float* xn, float* xk, bool normalize);
// Cap records (value, cell plane) of cap values in FFT-bin order.
int launch_cap_pack(tdm_ctx* c, const float2* caps, int n, CapRecs recs);
// One projected-gradient step with the TV gradient (steps tv_n, tv_k) and box constraints.
int launch_tv_step(tdm_ctx* c, const float* xn, const float* xk, const float* gn, const float* gk, float step,
                   float tv_n, float tv_k, float eps, float nlo, float nhi, float klo, float khi, float* xn_out,
                   float* xk_out);
// gather of the cap records rec (angles [0, n), specular positions posspec),
// normalisation and 3D inverse FFT into the outputs, on stream st.  Downloads
// run on c->dl_stream; each staged part (x-pass slab, counts, OTF) is
// rewritten only after the previous volume's download of that part is done
// (c->ev_dl).  ev_gathered (may be null) is recorded on st once the gather
// has read rec.
int launch_volume(tdm_ctx* c, int n, const VolumeOut& out, cudaStream_t st, CapRecs rec, const int2* posspec,
                  cudaEvent_t ev_gathered);
}  // namespace tdm
