/*
 * shwfs.h -- C ABI of the GB300 Shack-Hartmann wavefront-sensor engine.
 *
 * Drop-in native boundary for the reference's per-frame WFS step, the
 * Python extension ``cmod.cent`` built from cmod/src/centmodule.c and wrapped
 * by util/centcmod.py.  Each entry point below names the reference function it
 * replaces.  Signatures use plain pointers, sizes and status codes only; no
 * Python, numpy or torch types cross this boundary.
 *
 * Arrays are described by ``shwfs_array`` (float32 or int32, C-contiguous).
 * Like the reference, the phase input and the ``cents``/``bimg`` outputs are
 * BORROWED: the engine keeps the pointers and reads/writes them on every
 * run (cmod/src/centmodule.c:2934,3055-3058).  They may be host memory
 * (copied to/from the GPU inside run) or CUDA device memory (used in place).
 * Every other array is copied into device memory at initialise/update time,
 * so a caller that edits one of them in place must call shwfs_update again.
 *
 * All calls return a shwfs_status; SHWFS_OK is 0.  shwfs_last_error() returns
 * the message of the most recent failure on the calling thread.
 */
#ifndef SHWFS_H
#define SHWFS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum shwfs_status {
  SHWFS_OK = 0,
  SHWFS_ERR_INVALID = 1,     /* bad argument: shape, dtype, value */
  SHWFS_ERR_UNSUPPORTED = 2, /* valid in the reference, not implemented here */
  SHWFS_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  SHWFS_ERR_NOMEM = 4,       /* device or host allocation failed */
  SHWFS_ERR_STATE = 5        /* call not valid in the handle's current state */
} shwfs_status;

/* update codes: identical values to util/centcmod.py:19-40 and
 * cmod/src/centmodule.c:109-130 */
enum {
  SHWFS_CALSOURCE = 1,
  SHWFS_SIG = 2,
  SHWFS_ADDPOISSON = 3,
  SHWFS_NCEN = 4,
  SHWFS_READNOISE = 5,
  SHWFS_READBG = 6,
  SHWFS_NOISEFLOOR = 7,
  SHWFS_SKYBRIGHTNESS = 8,
  SHWFS_PXLPOWER = 9,
  SHWFS_SPOTPSF = 10,
  SHWFS_NTHREADS = 11,
  SHWFS_OPTICALBINNING = 12,
  SHWFS_CENTWEIGHT = 13,
  SHWFS_CORRELATIONCENTROIDING = 14,
  SHWFS_CORRTHRESH = 15,
  SHWFS_CORRPATTERN = 16,
  SHWFS_CALDATA = 17,
  SHWFS_REFCENTS = 18,
  SHWFS_CALCOEFF = 19,
  SHWFS_USEBRIGHTEST = 20,
  SHWFS_INTEGSTEPS = 21,
  SHWFS_OUTPUTPHASEARR = 22,
  /* extension (no reference counterpart): noise generator selection,
   * ival = SHWFS_NOISE_COUNTER or SHWFS_NOISE_REFERENCE */
  SHWFS_NOISEMODE = 100,
  /* extension: subapertures per CTA tile of the fused kernel, ival = 0 picks
   * the default for the geometry */
  SHWFS_TILESUBAPS = 101,
  /* extension: compute form, ival = SHWFS_FORM_* */
  SHWFS_FORM = 102,
  /* extension: zero-copy host I/O of shwfs_run/shwfs_run_async, ival = an
   * OR of SHWFS_HOSTIO_* (default: both) */
  SHWFS_HOSTIO = 103,
  /* extension: how sub-exposures (nintegrations > 1) form the image, ival =
   * SHWFS_INTEG_COMPAT (default) or SHWFS_INTEG_PHYSICAL */
  SHWFS_INTEGMODE = 104,
  /* extension: the tensor-core forms' GEMM staging, ival = an index into the
   * stagings that fit the handle's geometry (0 = the default choice;
   * shwfs_info.gemm_candidates gives their number); shwfs_autotune sets it
   * to the fastest.  Results do not depend on it.  Reset to 0 when the form
   * or the spot PSF changes. */
  SHWFS_GEMMSTAGING = 105
};

/* integration modes (SHWFS_INTEGMODE) */
enum {
  /* the reference's behaviour: the image accumulator is zeroed on every
   * sub-exposure (cmod/src/centmodule.c:478), so only the readout frame's
   * phase reaches the image */
  SHWFS_INTEG_COMPAT = 0,
  /* every exposed sub-exposure (the reference's start, middle and readout
   * frames; frame-transfer frames are not exposed) forms its normalised,
   * sky-added image on the device; the readout frame's image is their mean,
   * to which shot noise, read noise, threshold and centroiding are applied
   * once.  The total signal per readout stays sig.  Not available with
   * phase interpolation, phase+amplitude input or optical binning. */
  SHWFS_INTEG_PHYSICAL = 1
};

/* zero-copy host I/O switches (SHWFS_HOSTIO).  They apply to host arrays
 * that are pinned (the engine pins borrowed host arrays when it can) with
 * counter-based noise and no correlation centroiding; results are identical
 * either way, only the transfers change. */
enum {
  /* the kernels write the centroids and the final images of the lit
   * subapertures straight into the caller's host arrays, during the kernels,
   * instead of device copies followed by host copies */
  SHWFS_HOSTIO_OUTPUTS = 1,
  /* the image-formation kernels read the phase from the caller's host array
   * instead of a host-to-device copy ahead of them */
  SHWFS_HOSTIO_PHASE = 2
};

/* compute forms */
enum {
  SHWFS_FORM_FP32 = 0,   /* fused FP32 kernel, register FFTs (default) */
  SHWFS_FORM_BF16 = 1,   /* GEMM-DFT on tcgen05 tensor cores, one bf16 pass */
  SHWFS_FORM_BF16X3 = 2, /* GEMM-DFT, bf16 split products hi*hi + hi*lo + lo*hi */
  SHWFS_FORM_FP16 = 3,   /* GEMM-DFT, one fp16 pass, |F|^2 scaled per subaperture */
  SHWFS_FORM_TF32 = 4    /* GEMM-DFT, one tf32 pass (kind::tf32) */
};

/* noise generators */
enum {
  /* default: counter-based Philox4x32-10 streams keyed by (seed, frame,
   * subaperture, pixel); fully parallel; matches the reference in
   * distribution, not draw for draw */
  SHWFS_NOISE_COUNTER = 0,
  /* the reference's own streams: one PCG32 (Poisson) and one MT19937
   * (read noise) per reference worker thread, seeded seed+t, walking the
   * same static subaperture partition (cmod/src/centmodule.c:2535-2563) */
  SHWFS_NOISE_REFERENCE = 1
};

enum { SHWFS_F32 = 0, SHWFS_I32 = 1 };

typedef struct shwfs_array {
  const void* data; /* NULL means None */
  int ndim;
  int64_t shape[4];
  int dtype;     /* SHWFS_F32 or SHWFS_I32 */
  int on_device; /* 1: CUDA device pointer; 0: host pointer */
} shwfs_array;

/* The 41 positional arguments of cmod.cent.initialise
 * (cmod/src/centmodule.c:2876-2883, util/centcmod.py:115), in order.
 * ``sig`` and ``skybrightness`` are either scalars or arrays: a non-NULL
 * ``sigArr.data`` / ``skybrightnessArr.data`` selects the array form. */
typedef struct shwfs_init {
  int nthreads;
  int nsubaps;
  int ncen;
  int fftsize;
  int clipsize;
  int nimg;
  int phasesize;
  float readnoise;
  float readbg;
  int addPoisson;
  float noiseFloor;
  double sig;
  shwfs_array sigArr; /* float32 (nsubaps,) */
  double skybrightness;
  shwfs_array skybrightnessArr; /* float32 (nsubaps, nimg, nimg) */
  int calsource;
  float pxlPower;
  int nintegrations;
  int nlatency;
  uint64_t seed;
  shwfs_array phs;    /* float32 (W, W) phase or (2, W, W) phase + amplitude */
  shwfs_array pupfn;  /* float32 (nsubx, nsubx, p, p) */
  shwfs_array spotpsf; /* None, float32 (P, P) or (nsubx, nsubx, P, P) */
  shwfs_array cents;  /* float32 output, nsubaps*2 values */
  shwfs_array subflag; /* int32 (nsubx, nsubx) */
  shwfs_array bimg;   /* float32 output (nsubx, nsubx, nimg, nimg) */
  shwfs_array fracSubArea; /* float32 (nsubx, nsubx) */
  int opticalBinning;
  shwfs_array centWeight; /* None, float32 (corr, corr) or (nsubx, nsubx, corr, corr) */
  int correlationCentroiding;
  float corrThresh;
  shwfs_array corrPattern;
  shwfs_array corrimg;
  int threshType;
  int imageOnly;
  int useBrightest;
  shwfs_array useBrightestArr; /* None or int32 (nsubaps,) */
  int preBinningFactor;
  int parabolicFit;
  int gaussianFit;
  float gaussianMinVal;
  float gaussianReplaceVal;
  shwfs_array inputImage;
  shwfs_array subapLocation;
} shwfs_init;

/* value passed to shwfs_update */
enum {
  SHWFS_VAL_NONE = 0,
  SHWFS_VAL_INT = 1,
  SHWFS_VAL_FLOAT = 2,
  SHWFS_VAL_ARRAY = 3,
  SHWFS_VAL_TUPLE3 = 4 /* (calData, calBounds, calSteps) for SHWFS_CALDATA */
};
typedef struct shwfs_value {
  int kind;
  int64_t ival;
  double dval;
  shwfs_array arr[3];
} shwfs_value;

typedef struct shwfs_info {
  int nsubx, nsubaps, nlit;
  int fftsize, psfsize, clipsize, nimg, phasesize;
  int tile_subaps;      /* subapertures per CTA tile of the fused kernel */
  int smem_bytes;       /* dynamic shared memory per CTA */
  int grid_ctas;        /* CTAs launched per frame */
  int noise_mode;
  int cur_integ;
  uint64_t frames_read; /* readout frames processed (noise counter) */
  int form;             /* requested SHWFS_FORM_* */
  int form_active;      /* form the next readout will use (GEMM forms fall back to
                           FP32 for 4-D PSFs, phase+amplitude, optical binning,
                           reference-stream noise or sizes beyond the GEMM kernel) */
  int host_io_direct;   /* zero-copy host I/O of the last readout: 1 centroids and
                           2 images written into the host arrays by the kernels,
                           4 input (phase or detector image) read from the host
                           array by the kernels */
  int gemm_kcb;         /* tensor-core forms' staging: bytes of K per W2 chunk row, */
  int gemm_nw;          /* W2 ring stages, */
  int gemm_nk;          /* Kc ring stages, */
  int gemm_dbuf;        /* 1: two field buffers, 2: two |F|^2 buffers (OR), */
  int gemm_cw;          /* complex outputs per GEMM1 chunk; all 0 when no
                           tensor-core form is built */
  int gemm_staging;     /* index of the staging in use (SHWFS_GEMMSTAGING) */
  int gemm_candidates;  /* stagings that fit (0 without a tensor-core form) */
} shwfs_info;

typedef struct shwfs_handle shwfs_handle;

/* cmod.cent.initialise: py_initialise, cmod/src/centmodule.c:2858-3161.
 * Validates like the reference and uploads the constants. */
shwfs_status shwfs_initialise(const shwfs_init* init, shwfs_handle** out);

/* cmod.cent.run: py_run, cmod/src/centmodule.c:3188-3229.  One frame through
 * the integration state machine; blocks until cents/bimg are written;
 * *elapsed_s (may be NULL) receives the wall time in seconds. */
shwfs_status shwfs_run(shwfs_handle* h, float* elapsed_s);

/* cmod.cent.runSlope: py_runSlope, cmod/src/centmodule.c:3230-3272. */
shwfs_status shwfs_run_slope(shwfs_handle* h, float* elapsed_s);

/* cmod.cent.update: py_update, cmod/src/centmodule.c:2573-2856. */
shwfs_status shwfs_update(shwfs_handle* h, int code, const shwfs_value* val);

/* cmod.cent.free: py_free, cmod/src/centmodule.c:3163-3186. */
shwfs_status shwfs_free(shwfs_handle* h);

/* cmod.cent.testcorrelation: py_testcorrelation, cmod/src/centmodule.c:
 * 3275-3309.  img and corr are n x n float32 host arrays; corr holds a
 * half-complex pattern (what correlation mode 1 takes) and is replaced by
 * the correlation of img with it (calcCorrelation with corrsize = nimg = n,
 * unnormalised).  Runs on the current device and waits for the result. */
shwfs_status shwfs_test_correlation(int n, const float* img, float* corr);

/* Message of the last failure on this thread ("" if none). */
const char* shwfs_last_error(void);

/* ---- extensions (no reference counterpart) ---- */

/* shwfs_run without the final synchronisation: work is queued on ``stream``
 * (a cudaStream_t; NULL = the handle's own stream).  Host outputs are valid
 * once the stream has drained. */
shwfs_status shwfs_run_async(shwfs_handle* h, void* stream);

/* One readout frame from caller-supplied pre-noise images ("noise
 * injection"; no reference counterpart).  ``images`` holds, for every
 * subaperture, the image centroidsFromPhase has just before poissonise:
 * normalised, sky added (cmod/src/centmodule.c:1864-1872), float32
 * nsubaps*nimg*nimg, host or device memory.  The engine then runs the rest
 * of the readout as shwfs_run does -- shot noise, read noise, background
 * and threshold (:1879-1881), brightest pixels, pixel power, correlation,
 * centroids, calibration, references (:1882-1963), unlit subapertures
 * (:1964-1981) -- and writes cents/bimg; the integration state is neither
 * consulted nor advanced.
 * shot and readn (each NULL, or a shwfs_array of the same shape and type):
 *   both NULL  -- the handle's noise generator draws (SHWFS_NOISE_REFERENCE:
 *                 the reference's per-thread PCG32/MT19937 streams, so the
 *                 result equals the reference's noisy frame for the same
 *                 pre-noise images, seed and nthreads);
 *   otherwise  -- caller-drawn noise: shot[k] is used as the Poisson draw of
 *                 pixel k wherever the reference poissonises (addPoisson,
 *                 no calibration source, lit subaperture with light or sky),
 *                 readn[k] as the value of (float)gsl_ran_gaussian(r,
 *                 readNoise) wherever readCCD draws (readNoise != 0, no
 *                 calibration source, lit subapertures and, with imageOnly,
 *                 unlit ones).  An array the configuration draws from must
 *                 be given; the other may be NULL.
 * Rejected: optical binning and phase+amplitude handles
 * (SHWFS_ERR_UNSUPPORTED).  Blocks until the outputs are written. */
shwfs_status shwfs_run_prenoise(shwfs_handle* h, const shwfs_array* images, const shwfs_array* shot,
                                const shwfs_array* readn, float* elapsed_s);

/* Independent readout frames in one launch, all pointers device memory:
 * phase frames ``phs + f*phs_frame_stride`` (elements), outputs
 * ``cents + f*nsubaps*2`` and ``bimg + f*nsubaps*nimg*nimg``.  The
 * integration state is not consulted or advanced; the noise frame counter
 * advances by nframes. */
shwfs_status shwfs_run_batch(shwfs_handle* h, int nframes, const float* phs, int64_t phs_frame_stride,
                             float* cents, float* bimg, void* stream);

/* Rebind the borrowed phase / output arrays (same shapes as at initialise). */
shwfs_status shwfs_set_io(shwfs_handle* h, const shwfs_array* phs, const shwfs_array* cents,
                          const shwfs_array* bimg);

shwfs_status shwfs_get_info(const shwfs_handle* h, shwfs_info* info);

/* Library version string. */
const char* shwfs_version(void);

/* ---- many wavefront sensors per launch (no reference counterpart; the
 * reference serves several WFSs by resource sharing through one module
 * object, science/wfscent.py:41-52,585-598) ----
 * A batch captures one readout frame of every handle into a CUDA graph: each
 * handle's persistent kernel(s) on its own graph branch, branches running
 * concurrently, so WFSs of different subaperture counts, FFT sizes and spot
 * PSFs go to the GPU with one graph launch.  With shwfs_batch_set_multi,
 * handles on the fused FP32 kernel that share its (fftsize, psfsize)
 * instantiation and shared-memory footprint (counter noise, no correlation
 * centroiding, no phase interpolation) run as one persistent multi-handle
 * kernel over their tiles (up to 8 handles per launch) on a branch of its
 * own; results are identical either way.  Every handle must have
 * device-resident phs/cents/bimg.
 * The graph is re-captured when a handle is updated; noise frame counters
 * advance on the device between replays. */
typedef struct shwfs_batch shwfs_batch;
shwfs_status shwfs_batch_create(shwfs_handle* const* handles, int n, shwfs_batch** out);
shwfs_status shwfs_batch_run(shwfs_batch* b, void* stream);
shwfs_status shwfs_batch_free(shwfs_batch* b);
/* on != 0: group handles into multi-handle fused-kernel launches (off by
 * default: on the measured workloads the concurrent per-handle launches were
 * as fast or faster); re-captures the graph */
shwfs_status shwfs_batch_set_multi(shwfs_batch* b, int on);
/* multi-handle fused-kernel launches in the batch's captured graph */
shwfs_status shwfs_batch_multi_launches(const shwfs_batch* b, int* n);

/* Time the handle's phase-input kernels over their launch shapes on scratch
 * buffers and keep the fastest: for the FP32 form the candidate tile sizes
 * of the fused kernel (*best_tile receives the one kept); for a tensor-core
 * form every staging of the GEMM kernel that fits (GEMM1 output-chunk width,
 * W2 chunk width, double buffering of the field and |F|^2 operands, Kc
 * stages, W2 ring depth; shwfs_info.gemm_* report the one kept).  Results are
 * unchanged: the tile size only groups subapertures per CTA, and the MMAs
 * see the same k-steps in the same order whatever the staging. */
shwfs_status shwfs_autotune(shwfs_handle* h, int* best_tile);

/* fields of one row of shwfs_gemm_stagings */
enum {
  SHWFS_STG_CW = 0,     /* complex outputs per GEMM1 output chunk (GEMM1 N = 2 CW) */
  SHWFS_STG_NOC = 1,    /* GEMM1 output chunks covering the crop */
  SHWFS_STG_KCB = 2,    /* GEMM1 K bytes per row of one streamed W2 chunk */
  SHWFS_STG_NKC = 3,    /* W2 chunks per output chunk */
  SHWFS_STG_DBE = 4,    /* 1: two field (GEMM1 A) buffers */
  SHWFS_STG_DBA2 = 5,   /* 1: two |F|^2 (GEMM2 A) buffers */
  SHWFS_STG_NK = 6,     /* Kc (GEMM2 B) ring stages */
  SHWFS_STG_NW = 7,     /* W2 (GEMM1 B) ring stages */
  SHWFS_STG_ND1 = 8,    /* GEMM1 accumulator buffers in tensor memory */
  SHWFS_STG_K1 = 9,     /* GEMM1 K in elements */
  SHWFS_STG_N2 = 10,    /* GEMM2 N (nimg^2 rounded up to 16) */
  SHWFS_STG_SMEM = 11,  /* dynamic shared memory of a CTA, bytes */
  SHWFS_STG_TMEM = 12,  /* tensor-memory columns used (end of the last accumulator) */
  SHWFS_STAGING_FIELDS = 13
};

/* Host-only query (no GPU, no handle; no reference counterpart): the
 * stagings of the GEMM kernel that fit for tensor-core form `form`
 * (SHWFS_FORM_BF16 .. SHWFS_FORM_TF32), phasesize p, a crop x crop power
 * spectrum (the smaller of fftsize and the padded size: clipsize, or the
 * fftsize when pre-binning) and nimg x nimg
 * images, the default first, in the order SHWFS_GEMMSTAGING indexes them.
 * *n receives their number (0: the form cannot take this geometry and a
 * handle keeps the FP32 form); the first min(*n, cap) are written to rows,
 * SHWFS_STAGING_FIELDS ints each. */
shwfs_status shwfs_gemm_stagings(int form, int phasesize, int crop, int nimg, int* rows, int cap, int* n);

/* Timing aid (no reference counterpart): with a non-NULL CUDA event, every
 * readout of a tensor-core form records it on the launch stream between the
 * image-formation kernel and the noise/centroid kernel, so that a caller can
 * time the two separately.  NULL switches it off.  The event must outlive its
 * use by the handle. */
shwfs_status shwfs_set_split_event(shwfs_handle* h, void* event);

/* Draws of the engine's counter-based noise for testing its samplers (no
 * reference counterpart; the reference draws through rk_poisson/gsl,
 * cmod/src/centmodule.c:722-784).  Element i is drawn as the pipeline draws
 * pixel i & 0xffff of subaperture i >> 16 in frame `frame`: kind 2 out[i] ~
 * Poisson(lam[i]) by the tabulated sampler every compute form uses (the
 * pixel's quad stream below lambda 64, PTRS from its own stream above);
 * kind 1 out[i] ~ N(0, 1), the pixel's read-noise normal (lam unused);
 * kind 0 out[i] ~ Poisson(lam[i]) by the table-free modal inversion from a
 * stream of its own (an independent exact sampler, kept to cross-check
 * kind 2).  lam and out are device pointers; with stream NULL the call waits
 * for the result. */
shwfs_status shwfs_sample_noise(int kind, const float* lam, int64_t n, uint64_t seed, uint64_t frame, float* out,
                                void* stream);

/* ---- infinite phase screen on the device (science/infScrn.py) ----
 *
 * A screen of ny x nx float32 phase values kept in HBM as a circular buffer.
 * shwfs_screen_add appends n columns (axis 0) or rows (axis 1) at the end,
 * each A Z + coeff_turb B noise (+ step on the first one), Z the last two
 * columns (rows) stacked oldest first, as addNewColumnOnEnd /
 * addNewRowOnEnd (science/infScrn.py:747-791, 825-855); the oldest column
 * (row) is dropped.  axis 2 (columns) and 3 (rows) add them at the start
 * instead, as addNewColumnOnStart / addNewRowOnStart (:793-823, 857-887)
 * with AStart, A's column blocks in reverse order (:722-731), on the first
 * two lines; the last column (row) is dropped.  ay (ny x 2ny), by (ny x ny), ax (nx x 2nx), bx
 * (nx x nx) are row-major float64 host arrays (either axis may be NULL if
 * never extruded); init is the initial screen (ny x nx, host).  noise: NULL
 * for the device's counter-based normals (seed, extrusion index), else n
 * host vectors of ny (nx) float64 normals to inject.  shwfs_screen_window
 * copies an h x w window at (y0, x0) of the current screen to a device
 * array (row stride out_stride) -- a WFS's phase, without a host copy.
 * With stream NULL the calls wait for the result. */
typedef struct shwfs_screen shwfs_screen;
shwfs_status shwfs_screen_create(int ny, int nx, const float* init, const double* ay, const double* by,
                                 const double* ax, const double* bx, uint64_t seed, shwfs_screen** out);
shwfs_status shwfs_screen_add(shwfs_screen* s, int axis, int n, double coeff_turb, double step, const double* noise,
                              void* stream);
shwfs_status shwfs_screen_window(shwfs_screen* s, int y0, int x0, int h, int w, float* out, int64_t out_stride,
                                 void* stream);
shwfs_status shwfs_screen_read(shwfs_screen* s, float* host_out);
/* Pupil phase from several layers for a source at infinity (createPupilPhs,
 * util/atmos.py:678-833, NGS path): layer q contributes the (npup+1)-square
 * window of screens[q] at logical (y0[q], x0[q]) shifted by linearshift
 * (cmod/src/interpmodule.c:1234-1300) with fractional shifts yshift[q]
 * (rows) and xshift[q] (columns) in [0, 1]; layers are added in order, the
 * piston sum(phase * pupil) / pupil_area is removed when remove_piston, and
 * the result is multiplied by the pupil and by scale (500 / wavelength in
 * the reference).  pupil and out are npup x npup device arrays; 1..16
 * layers.  With stream NULL the call waits for the result. */
shwfs_status shwfs_screens_pupil_phase(shwfs_screen* const* screens, int nlayers, const int* y0, const int* x0,
                                       const float* yshift, const float* xshift, int npup, const float* pupil,
                                       double pupil_area, int remove_piston, float scale, float* out, void* stream);
shwfs_status shwfs_screen_free(shwfs_screen* s);

/* ---- reconstructor step (science/tomoRecon.py:1077-1107, 1196-1223) ----
 *
 * act[i] = decay_i * act[i] - gain_i * sum_j R[i, j] x[j], R nacts x ncents
 * row-major float32; gains/decay per actuator (device arrays) or, when NULL,
 * the scalars gain/decay_scalar.  All arrays are device pointers; with
 * stream NULL the call waits for the result. */
shwfs_status shwfs_mvm_update(int nacts, int ncents, const float* R, const float* x, const float* gains, float gain,
                              const float* decay, float decay_scalar, float* act, void* stream);

/* Self-test of the pipeline's bounded waits (no counterpart in the
 * reference): a one-CTA kernel waits on an mbarrier that nothing arrives on,
 * for at most max_cycles SM clocks.  *timed_out = 1 when the wait gave up
 * and *abort_raised = 1 when it raised the CTA's abort flag, as every
 * tensor-core pipeline wait does before the kernel drains and the handle
 * reports SHWFS_ERR_STATE.  Returns after the kernel has finished; the
 * context stays usable. */
shwfs_status shwfs_selftest_bounded_wait(int64_t max_cycles, int* timed_out, int* abort_raised);

/* ---- allocation-free image centroiding (no counterpart in the reference) ----
 *
 * For callers that cannot allocate GPU memory: a real-time control thread
 * that must never call cudaMalloc/cudaFree while it runs (an allocation may
 * wait for the whole device to synchronise), or an application whose device
 * memory is all owned by its own allocator.  Such callers cannot create a
 * shwfs handle, which allocates device copies of its configuration.
 *
 * shwfs_image_centroids_noalloc cuts the nsubx x nsubx subaperture images
 * out of a detector image (2-D, tiled by nimg, or 4-D nsubx,nsubx,nimg,nimg),
 * thresholds them and computes centre-of-gravity centroids, exactly as
 * shwfs_run_slope does for a handle with the same settings and no
 * subapLocation.  Every array is caller-owned device memory; the call
 * allocates nothing.  Its only working memory (the lit/unlit subaperture
 * lists) is a static device array of SHWFS_NOALLOC_MAX_SUBAPS entries each,
 * about 512 KB held on every GPU that loads the library until the process
 * exits; larger sensors are rejected with SHWFS_ERR_INVALID.
 *
 * The first call on a device looks up that array's device address (once per
 * device); make that first call before any stream capture.  Every call
 * synchronises ``stream`` once, to read the subaperture counts back to the
 * host before it launches the centroiding kernels.  All calls share the one
 * array, which keeps the last call's contents (each call rebuilds what it
 * reads), so calls whose GPU work overlaps -- other streams, other host
 * threads -- race and must not be issued.  ``err`` (may be NULL) receives a
 * message on failure. */
#define SHWFS_NOALLOC_MAX_SUBAPS 65536
typedef struct shwfs_image_job {
  int nsubx, nimg, ncen;
  int image_ndim;        /* 2: (image_rows, image_cols) detector image; 4: (nsubx,nsubx,nimg,nimg) */
  int64_t image_rows, image_cols;
  const float* image;    /* device */
  const int* subflag;    /* device, int32, nsubx*nsubx: 1 = subaperture used */
  const float* refCents; /* device, nsubx*nsubx*2 reference centroids, or NULL */
  float noiseFloor;
  int threshType;
  int calsource;
  int useBrightest;
  float pxlPower;
  int imageOnly;         /* 1: images only, unused subapertures get read noise */
  float readNoise, readBg;
  uint64_t seed, frame;  /* counter-based read-noise stream for imageOnly */
  float* cents;          /* device output, nsubx*nsubx*2 */
  float* bimg;           /* device output, nsubx*nsubx*nimg*nimg */
} shwfs_image_job;
shwfs_status shwfs_image_centroids_noalloc(const shwfs_image_job* job, void* stream, char* err, size_t errlen);

/* ---- serving loop (no reference counterpart; the reference runs each WFS
 * of a simulation in its own process step, science/wfscent.py:585-683) ----
 * A server owns a dispatcher thread that serves WFS-frame requests of many
 * simulated AO systems on one GPU with continuous batching: a request is
 * launched as soon as its release time has passed, its system has no frame
 * in flight and a device slot is free, each system on its own CUDA stream so
 * that frames of different systems overlap on the device.  Systems are
 * admitted against a fixed HBM budget: a system whose device state does not
 * fit waits until removed systems free enough memory.  A system's state
 * (pupil, PSF spectra, tables, integration state, output buffers) stays on
 * the device while it is admitted.  The engine of a system is created from
 * its shwfs_init when admitted; the arrays the init points to must stay
 * valid until then (phs, cents and bimg there only give shapes: the server
 * allocates the system's own device buffers).  All calls are thread-safe. */
typedef struct shwfs_server shwfs_server;
typedef struct shwfs_server_config {
  int64_t hbm_budget_bytes; /* device memory the admitted systems may hold */
  int max_inflight;         /* frames on the device at once (all systems) */
  int device;               /* CUDA device ordinal */
  int integration_mode;     /* SHWFS_INTEG_* for every system (0: the reference's) */
} shwfs_server_config;
typedef struct shwfs_completion {
  uint64_t request;  /* id returned by shwfs_server_submit */
  int system;
  int status;        /* SHWFS_OK, or the failure of this frame */
  int readout;       /* 1: a readout frame (centroids written), 0: integrating */
  double latency_s;  /* from the release time to completion seen by the server */
  double done_s;     /* completion time on the server clock */
} shwfs_completion;
typedef struct shwfs_server_stats {
  int systems, admitted, pending;
  int64_t used_bytes, budget_bytes;
  int inflight;
  uint64_t submitted, completed;
} shwfs_server_stats;

shwfs_status shwfs_server_create(const shwfs_server_config* cfg, shwfs_server** out);
/* form: SHWFS_FORM_*; *system receives the system id */
shwfs_status shwfs_server_add_system(shwfs_server* s, const shwfs_init* init, int form, int* system);
shwfs_status shwfs_server_remove_system(shwfs_server* s, int system);
/* One WFS frame of `system` from the W x W float32 phase at `phs` (device
 * pointer when phs_on_device, else host); released at release_s on the
 * server clock (seconds since creation; <= 0: now).  With out_cents non-NULL
 * the frame's centroids (nsubaps*2 floats, host memory) are written there
 * before the completion is reported.  The phase must stay valid until the
 * request completes. */
shwfs_status shwfs_server_submit(shwfs_server* s, int system, const float* phs, int phs_on_device, float* out_cents,
                                 double release_s, uint64_t* request);
/* up to max completions since the last poll; *n receives the count */
shwfs_status shwfs_server_poll(shwfs_server* s, shwfs_completion* out, int max, int* n);
shwfs_status shwfs_server_get_stats(shwfs_server* s, shwfs_server_stats* st);
/* seconds since the server was created */
double shwfs_server_clock(shwfs_server* s);
shwfs_status shwfs_server_destroy(shwfs_server* s);

#ifdef __cplusplus
}
#endif
#endif /* SHWFS_H */
