/*
 * tdm.h — C ABI of the GB300 tomographic diffractive microscopy hot path.
 *
 * Drop-in for the two batch programs of madeba/MTD_transmission:
 *   tomo_pretraitement   (Tomo_prog/pretraitement_hors_axe_CPU/main.cpp)
 *   tomo_reconstruction  (Tomo_prog/Reconstruction/main.cpp)
 * The reference has no library interface; these entry points are its
 * function-level seams, each citing the reference code it replaces.  The
 * executables tomo_pretraitement / tomo_reconstruction / tomo_pipeline built
 * from this library keep the reference's file contracts.
 *
 * Conventions
 *  - Every pointer argument may be host memory (pageable or pinned) or device
 *    memory of the context's GPU; the library detects which.  Calls whose
 *    buffers are all device memory are asynchronous on the context's stream
 *    (tdm_stream); calls that touch host memory return after the results are
 *    in host memory.
 *  - Complex arrays are interleaved float pairs (re, im), row-major with x
 *    fastest, as the reference's std::vector<std::complex<double>> with
 *    cpt = x + y*dim (+ z*dim*dim).
 *  - posspec arrays hold n x-coordinates followed by n y-coordinates (the
 *    layout of tab_posSpec.raw, main.cpp:250-251), as int32.
 *  - Return value: TDM_OK (0) or a negative TDM_E* status; tdm_last_error()
 *    gives the message.  One context per host thread.
 */
#ifndef TDM_H
#define TDM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TDM_OK 0
#define TDM_EINVAL -1       /* invalid argument */
#define TDM_EUNSUPPORTED -2 /* geometry outside what the kernels support */
#define TDM_ECUDA -3        /* CUDA runtime error */
#define TDM_ENOMEM -4       /* device allocation failed */
#define TDM_EDATA -5        /* data error (fit undefined, cap voxel outside the volume) */
#define TDM_EIO -6          /* file input/output error */

typedef struct tdm_ctx tdm_ctx;

/* Acquisition and reconstruction parameters: the keys of recon.txt and
 * config_manip.txt that the path reads (pretraitement_hors_axe_CPU/manip.cpp:32-104,
 * Reconstruction/src/manip.cpp:44-94).  Real-valued keys carry the value the
 * reference's extract_val returns, i.e. rounded to float
 * (pretraitement_hors_axe_CPU/src/IO_fonctions.cpp:81-118). */
typedef struct {
    int ccd_roix;       /* CCD_ROIX: hologram side H (power of two, 256..2048) */
    int nxmax;          /* NXMAX: N; fields are F = 2N square (F power of two, 64..512) */
    int circle_cx;      /* CIRCLE_CX: +1 order centre in the fftshifted hologram spectrum */
    int circle_cy;      /* CIRCLE_CY */
    int dim_final;      /* DIM_FINAL: D, volume side (power of two, >= 4N, <= 1024) */
    int born;           /* BORN: 1 Born, 0 Rytov */
    int c_aber;         /* C_ABER: aberration correction (and unwrapping) on/off */
    int deroul;         /* DEROUL: phase unwrapping on/off (only with C_ABER) */
    int volkov;         /* VOLKOV: 1 Volkov; 0 Herraez (tdm_create then draws the C library's
                           rand() sequence as the reference would for max_angles angles:
                           max_angles * (2*NXMAX)^2 draws, about 60 ms for 600 x 256^2) */
    double na;          /* NA */
    double n0;          /* N0 */
    double lambda0;     /* LAMBDA (m) */
    double f_tube;      /* F_TUBE (m) */
    double f_obj;       /* F_OBJ (m) */
    double tpcam;       /* TPCAM (m) */
    double rf;          /* RF */
    double coef_na_obj_limit; /* COEF_NA_OBJ_LIMIT (recon.txt, default 1) */
} tdm_geom;

/* Derived quantities (pretraitement_hors_axe_CPU/manip.cpp:43-57,104;
 * Reconstruction/src/manip.cpp:64-94). */
typedef struct {
    double rayon;       /* Ewald radius in spectrum pixels, round(NXMAX*n0/NA) */
    double tp_holo;     /* tailleTheoPixelHolo (m) */
    double tp_uborn;    /* tailleTheoPixelUborn (m) */
    double tp_tomo;     /* tailleTheoPixelTomo (m) */
    double delta_f;     /* Delta_fUborn (1/m) */
} tdm_derived;

/* Creates a context on the current CUDA device for stacks of up to
 * max_angles holograms (TDM_EUNSUPPORTED above 65535, or above what the cap
 * gather's per-CTA angle list allows for the geometry: 24,620 angles at
 * NXMAX 128, DIM_FINAL 512; the limit is printed on stderr).  A context is
 * used by one host thread at a time.  Replaces the FFTW plan set-up of both programs
 * (pretraitement_hors_axe_CPU/main.cpp:91-105,180-189; Reconstruction/main.cpp:131,185,318). */
int tdm_create(const tdm_geom* geom, int max_angles, tdm_ctx** out);
/* Releases the context and its device memory (no counterpart: the reference's
 * programs exit without releasing their plans). */
int tdm_destroy(tdm_ctx* ctx);
const char* tdm_last_error(const tdm_ctx* ctx);
/* Derived quantities of the context's geometry, and without a context (host
 * arithmetic only): the manip constructors' derived members
 * (pretraitement_hors_axe_CPU/manip.cpp:43-57,104; Reconstruction/src/manip.cpp:64-94). */
int tdm_get_derived(const tdm_ctx* ctx, tdm_derived* out);
int tdm_derive(const tdm_geom* geom, tdm_derived* out);

/* Aberration mask, F*F uint8 (Image_mask.pgm); NULL selects the unit mask.
 * Replaces init_mask_aber, countM, initCorrAber
 * (pretraitement_hors_axe_CPU/Correction_aberration.cpp:36-149; main.cpp:192-208). */
int tdm_set_mask(tdm_ctx* ctx, const uint8_t* mask);

/* Reference intensity, H*H float (the Intensite_ref.pgm image of the ROI, host
 * or device memory), or NULL to clear it.  While set, every hologram pixel is
 * divided by the reference amplitude sqrt(I_ref) (1 where I_ref is 0) before
 * the extraction.  Replaces initRef (pretraitement_hors_axe_CPU/fonctions.cpp:46-61)
 * and the division of main.cpp:147.  Off by default, as in the reference,
 * where those lines are commented out (main.cpp:109,147). */
int tdm_set_reference_intensity(tdm_ctx* ctx, const float* intensity);

/* Off-axis extraction of n holograms (H*H samples each, uint8 when bits == 8,
 * uint16 when bits == 16) into the context's spectrum stack; the F*F crops
 * are also copied to spectra_out (n*F*F complex) when it is not NULL.
 * Replaces holo2TF_UBorn (pretraitement_hors_axe_CPU/fonctions.cpp:279-304)
 * called from main.cpp:130-165. */
int tdm_extract(tdm_ctx* ctx, const void* holos, int bits, int n, float* spectra_out);

/* Field formation for n spectra: specular search, recentring and inverse FFT,
 * phase, Volkov unwrapping, aberration fits, Born/Rytov.  spectra_in NULL
 * uses the context's stack (from tdm_extract).  fields_out (n*F*F complex,
 * UBornFinal) and posspec_out (2n int32) may be NULL.
 * Replaces the second loop of tomo_pretraitement (pretraitement_hors_axe_CPU/main.cpp:230-342):
 * coordSpec (fonctions.cpp:88-101), calc_Uborn2 (:348-374),
 * calcPhase_mpi_pi_atan2 (:39-43), deroul_volkov4_total_sym_paire
 * (src/deroulement_volkov4.cpp:14-92), aberCorr2/ampliCorr2
 * (Correction_aberration.cpp:166-184). */
int tdm_fields(tdm_ctx* ctx, const float* spectra_in, int n, float* fields_out, int32_t* posspec_out);

/* Same as tdm_fields, also returning per-angle intermediates (each n*F*F
 * float, any may be NULL): wrapped phase, unwrapped phase, amplitude. */
int tdm_fields_debug(tdm_ctx* ctx, const float* spectra_in, int n, float* fields_out, int32_t* posspec_out,
                     float* phase_out, float* unwrapped_out, float* amp_out);

/* Reconstruction of the D^3 volume from n fields: per-field window, FFT and
 * shift, Ewald-cap mapping with hit counts, normalisation, OTF mask, 3D
 * inverse FFT and index conversion.  fields_in / posspec_in NULL use the
 * context's results of tdm_fields.  Outputs (D^3 each, index x + y*D + z*D*D,
 * any may be NULL): indice (real part, indice.tif), absorption (imaginary
 * part, absorption.tif), otf (OTF3D mask, 0/1), counts (sup_redon before its
 * zeros are replaced).
 * Replaces Reconstruction/main.cpp:203-352: decal2DCplxGen
 * (src/fonctions.cpp:1268-1309), TF2Dcplx (src/FFT_fonctions.cpp:333-349),
 * retroPropag_Born (src/fonctions.cpp:875-935), fftshift3D
 * (src/FFT_fonctions.cpp:78-151), TF3Dcplx_INV (:394-412). */
int tdm_reconstruct(tdm_ctx* ctx, const float* fields_in, const int32_t* posspec_in, int n, float* indice_out,
                    float* absorption_out, uint8_t* otf_out, uint32_t* counts_out);

/* Holograms to volume in one call, fields kept on the device (tomo_pipeline).
 * Equivalent to tdm_extract + tdm_fields + tdm_reconstruct.  Replaces the two
 * programs run back to back (pretraitement_hors_axe_CPU/main.cpp:31-363, then
 * Reconstruction/main.cpp:57-384) without the field files between them. */
int tdm_pipeline(tdm_ctx* ctx, const void* holos, int bits, int n, float* indice_out, float* absorption_out,
                 uint8_t* otf_out, uint32_t* counts_out, int32_t* posspec_out);

/* tdm_pipeline that returns once the work is queued, for a sequence of
 * volumes (time-lapse acquisition).  No counterpart in the reference.  Host
 * buffers should be page-locked (cudaHostAlloc / cudaHostRegister) for the
 * copies to run asynchronously, and must stay untouched until
 * tdm_synchronize(ctx) returns; the outputs are complete only then.  Calls on
 * one context run in order; a call's uploads and kernels overlap the
 * previous call's output downloads (separate copy engines). */
int tdm_pipeline_async(tdm_ctx* ctx, const void* holos, int bits, int n, float* indice_out, float* absorption_out,
                       uint8_t* otf_out, uint32_t* counts_out);

/* ---- Forward operator, adjoint and regularised reconstruction ----
 * No counterpart in the reference's built code: they are the operators of
 * the iterative constrained reconstruction its configuration keys describe
 * (recon.txt GERCHBERG, NB_ITER_GPS, DELTA_NMIN/MAX, KAPPA_MIN/MAX; the
 * tomo_GPS program itself is absent).  Volumes are D^3 float32 arrays in the
 * layout of tdm_reconstruct's outputs ([z][y][x], x fastest); x = index +
 * i absorption.  G(x) = M_in FFT3(M_out x) / (s D^3) is the exact inverse of
 * the reconstruction's volume stage (s its index scale, M the fftshift sign
 * patterns); S samples each angle's Ewald-cap cells (the cells
 * tdm_reconstruct accumulates, same geometry).  posspec: 2n ints (x values
 * then y values, host or device) or NULL for the context's specular
 * positions (from the last tdm_fields, tdm_pipeline or tdm_reconstruct call).
 * Pointers may be host or device memory. */

/* caps_out (n x F x F complex, FFT-bin order [angle][ky][kx], 0 outside the
 * caps) = S G(index + i absorption); absorption may be NULL (0). */
int tdm_forward(tdm_ctx* ctx, const float* index, const float* absorption, int n, const int32_t* posspec,
                float* caps_out);

/* Adjoint of tdm_forward: index_out + i absorption_out = G^H S^H caps (the
 * unnormalised scatter of the cap values into their cells, then G^H);
 * absorption_out may be NULL. */
int tdm_adjoint(tdm_ctx* ctx, const float* caps, int n, const int32_t* posspec, float* index_out,
                float* absorption_out);

typedef struct {
    int iterations;            /* projected-gradient iterations */
    int init;                  /* 0: start from index_io / absorption_io; 1: from the single-pass reconstruction */
    float step;                /* data step (1: each iteration makes the measured cells data-consistent) */
    float tv_weight;           /* TV gradient step per iteration, relative to each channel's box range
                                  (max - min; absolute when the box is unbounded); 0: no regularisation */
    float tv_eps;              /* TV smoothing: sum sqrt(|grad x|^2 + eps^2) */
    float index_min, index_max;            /* box constraints (DELTA_NMIN, DELTA_NMAX) */
    float absorption_min, absorption_max;  /* (KAPPA_MIN, KAPPA_MAX) */
} tdm_tv_opts;

typedef struct {
    int iterations;            /* iterations run */
    double misfit_first;       /* sum |S G x - caps|^2 at the first and the last iteration */
    double misfit_last;
    double seconds;            /* device time of the iterations */
} tdm_tv_report;

/* Regularised reconstruction: x <- clamp(x - step T(S^H (S G x - caps) / count)
 * - tv dTV(x)), tv = tv_weight x the box range, T = G^-1, count the cells' hit counts (the
 * single-pass reconstruction's normalisation as the preconditioner), the
 * clamp the box constraints.  caps: n x F x F complex cap values, or NULL
 * for the context's cap records (from the last tdm_pipeline or
 * tdm_reconstruct call: the measured fields' cap contributions).  index_io
 * (and absorption_io, or NULL to reconstruct the index alone) hold the
 * starting volume when opts->init = 0 and receive the result, so a run can
 * be continued from a saved iterate. */
int tdm_tv_reconstruct(tdm_ctx* ctx, const float* caps, int n, const int32_t* posspec, const tdm_tv_opts* opts,
                       float* index_io, float* absorption_io, tdm_tv_report* report);

/* ---- Batched acquisitions ----
 * Several stacks of uneven size (one context each, any geometries) processed
 * by one CUDA-graph launch.  No counterpart in the reference.
 * tdm_batch_create captures, for stack i, tdm_pipeline(ctxs[i], holos[i],
 * bits[i], n[i], indice[i], absorption[i], otf[i], NULL, NULL) into one
 * graph in which the stacks are independent branches; all buffers must be
 * device memory and are bound at creation (refill holos[i] between
 * launches).  tdm_batch_launch runs the graph on `stream` (a cudaStream_t,
 * 0 for the default stream) and returns without waiting.  A context must
 * not be used by other calls while a launch of a batch that holds it runs. */
typedef struct tdm_batch tdm_batch;
int tdm_batch_create(int count, tdm_ctx* const* ctxs, const void* const* holos, const int* bits, const int* n,
                     float* const* indice, float* const* absorption, uint8_t* const* otf, tdm_batch** out);
int tdm_batch_launch(tdm_batch* batch, void* stream);
int tdm_batch_destroy(tdm_batch* batch);

/* Off-axis extraction that allocates nothing.  No counterpart in the
 * reference: it is for callers that cannot allocate GPU memory, such as a
 * camera acquisition loop that must not stall on cudaMalloc between bursts of
 * frames, or a host application whose memory pool already owns the device.
 * Same result as tdm_extract on a context without a reference intensity
 * (tdm_set_reference_intensity is not applied here), without a context: holos
 * (n*H*H uint8/uint16, 2-byte aligned when 16-bit) and spectra_out (n*F*F
 * complex, 8-byte aligned) must be memory of the current device; the work runs on
 * `stream` (a cudaStream_t, 0 for the default stream) and the call returns
 * without waiting.  Scratch lives in a fixed 4 MiB array inside the library
 * (held by every GPU that loads it until exit): CCD_ROIX * 2*NXMAX may not
 * exceed 524288 (TDM_EUNSUPPORTED otherwise).  The first call on a device
 * looks up that array and uploads the twiddle and window tables; make it
 * before any stream capture.  All calls share the scratch, so calls that
 * overlap on the GPU (other streams or threads) race. */
int tdm_extract_noalloc(const tdm_geom* geom, const void* holos, int bits, int n, float* spectra_out, void* stream);

/* Planes of the D^3 spectrum that the Ewald caps can reach, [zmin, zmin +
 * band): the gather sums only these, and its z transform takes the other
 * planes as zero.
 * Diagnostic; no counterpart in the reference. */
int tdm_cap_planes(const tdm_ctx* ctx, int* zmin, int* band);

/* Bounded device waits (no counterpart in the reference; the reference has no
 * device code).  The extraction's row pass stages hologram rows with bulk
 * copies and waits for each at most `polls` polls (default and maximum 2^24;
 * a negative value restores the default) before it records an error; the
 * call's tdm_synchronize then returns TDM_ECUDA ("a bulk copy of hologram rows
 * did not complete").  After that first bound the warp still waits, up to the
 * default bound, for its copy, so no copy is left in flight.  0 makes every
 * first wait give up at once, which tests the error path without a fault.
 * Waits for the context's queued work first. */
int tdm_set_wait_limit(tdm_ctx* ctx, long long polls);

/* Schedule of the per-angle stages (no counterpart in the reference): tdm_pipeline
 * streams the angles in chunks of `chunk` and keeps `lanes` consecutive chunks in
 * flight at once, each on its own stream with its own scratch (1 <= lanes <= 8,
 * chunk * lanes <= min(128, max_angles rounded up to a multiple of 16), the
 * scratch capacity of the context).  Default: chunk 16, 4 lanes (fewer when the
 * capacity or the stack is smaller).  Waits for the context's queued work first.
 * Results do not depend on the schedule. */
int tdm_set_schedule(tdm_ctx* ctx, int chunk, int lanes);

/* Project autotuner (no counterpart in the reference): times tdm_pipeline on
 * the given stack (device holograms) with the schedules (chunk, lanes) = (16, 4),
 * (16, 2), (8, 4), (12, 4), (32, 2), (16, 6) and (32, 4) that fit the context's
 * scratch and keeps the fastest; *chunk_out receives its chunk. */
int tdm_autotune(tdm_ctx* ctx, const void* holos, int bits, int n, int* chunk_out);

/* Stream-ordered execution helpers.  tdm_pipeline queues each volume's stage
 * (gather, 3D inverse FFT, outputs) on a second stream of the context, so that
 * it overlaps the next call's per-angle stages; tdm_join orders the context
 * stream after those volume stages (the other entry points do this
 * themselves; tdm_synchronize waits for everything). */
int tdm_synchronize(tdm_ctx* ctx);
int tdm_join(tdm_ctx* ctx);
void* tdm_stream(tdm_ctx* ctx);               /* cudaStream_t of the context */
uint64_t tdm_launch_count(const tdm_ctx* ctx); /* kernels launched so far */
/* Device-side elapsed time of the last tdm_* call's dominant kernel group
 * (milliseconds per stage) for profiling: names are "extract", "fields",
 * "map", "volume"; returns a negative value for an unknown name.  After
 * tdm_pipeline, which streams extraction, fields and cap mapping chunk by
 * chunk, "extract" covers all three and "fields" and "map" read 0. */
double tdm_stage_ms(const tdm_ctx* ctx, const char* stage);

/* Opt-in per-kernel timing: when enabled, every kernel launch is bracketed by
 * a pair of CUDA events on the context stream.  tdm_profile() clears the
 * records; tdm_profile_read() waits for the stream and returns, for kernel
 * index 0 <= index < tdm_profile_count(), its name, the summed device time
 * and the number of launches since the last tdm_profile() call. */
int tdm_profile(tdm_ctx* ctx, int enable);
int tdm_profile_count(void);
int tdm_profile_read(tdm_ctx* ctx, int index, const char** name, double* total_ms, int* launches);

/* ---- Host-side file contract helpers (executables and tests) ---- */

/* extract_val: value of a KEY in a whitespace "KEY value" file, last
 * occurrence wins, '#' comment lines, float-rounded; def when absent
 * (pretraitement_hors_axe_CPU/src/IO_fonctions.cpp:81-118,
 * Reconstruction/src/fonctions.cpp:137-180).  Returns 1 when found, 0 when
 * absent, TDM_EIO when the file cannot be opened. */
int tdm_extract_val(const char* path, const char* key, double def, double* out);
/* extract_string (pretraitement_hors_axe_CPU/src/IO_fonctions.cpp:44-79). */
int tdm_extract_string(const char* path, const char* key, char* out, size_t cap);
/* Fills a tdm_geom from recon.txt and config_manip.txt, as the manip
 * constructors read them (pretraitement_hors_axe_CPU/manip.cpp:9-157,
 * Reconstruction/src/manip.cpp:10-163). */
int tdm_read_geom(const char* recon_txt, const char* config_manip_txt, tdm_geom* out);
/* Binary PGM (P5) reader, 8- or 16-bit (16-bit samples are big-endian in the
 * file).  Replaces charger_image2D_OCV (pretraitement_hors_axe_CPU/src/IO_fonctions.cpp:24-40)
 * with native sample depth: *bits is set to 8 or 16; the ROI is the top-left
 * roi x roi corner.  buf receives roi*roi samples (uint8 or uint16). */
int tdm_read_pgm(const char* path, int roi, void* buf, int* bits);
/* Size and maximum sample value of a PGM file (the image size that
 * charger_image2D_OCV takes from the decoded image,
 * pretraitement_hors_axe_CPU/src/IO_fonctions.cpp:26,32). */
int tdm_pgm_info(const char* path, int* width, int* height, int* maxval);
/* Float32 multi-page TIFF writer (SAV3D_Tiff_Optimized,
 * Reconstruction/src/fonctions.cpp:2286-2357, pages of dim_x x dim_y, resolution
 * 0.01/pixel_size per cm; BigTIFF beyond 4 GB).  orientation is the TIFF
 * Orientation tag: 4 (BOTLEFT) for the volumes, 1 (TOPLEFT) for the 2D images
 * of SAV_Tiff2D (pretraitement_hors_axe_CPU/src/IO_fonctions.cpp:364-400). */
int tdm_write_tiff_f32(const char* path, const float* vol, int dim_x, int dim_y, int pages, double pixel_size,
                       int orientation);

/* HDF5 file of a complex volume, as the polarisation mode of the reference's
 * reconstruction writes it (save_complex_volume_hdf5,
 * Reconstruction/src/IO_functions.cpp:52-82, called at Reconstruction/main.cpp:360-363):
 * group "/indice_complexe" with float32 datasets "Re" and "Im" of dimensions
 * (nz, ny, nx), x fastest in re and im.  A minimal writer of the HDF5 format
 * (superblock version 0, symbol-table groups, contiguous datasets); no
 * library. */
int tdm_write_hdf5_complex(const char* path, const float* re, const float* im, int nx, int ny, int nz);

#ifdef __cplusplus
}
#endif

#endif /* TDM_H */
