/*
 * cyrsoxs.h - C ABI of the GB300-native CyRSoXS scattering engine.
 *
 * Drop-in boundary for the per-energy, per-E-angle scattering path of
 * usnistgov/cyrsoxs v1.2.0.0.  Plain C types only: pointers, sizes and a
 * status code.  Errors never terminate the process (the reference calls
 * exit(); include/cudaHeaders.h:39-63); they return a non-zero status and
 * cyr_last_error() describes the failure.
 *
 * Array layouts (the reference's own, include/Input/Input.h:35-94,
 * src/cudaMain.cu:968-971):
 *   voxels      float[num_material][nz][ny][nx][4]  Voxel::s1 per material,
 *               Euler (S, theta, psi, Vfrac) or vector (sx, sy, sz, phi_unaligned)
 *   optical     float[num_energies][num_material][4] (delta_par, beta_par,
 *               delta_perp, beta_perp); n = 1 - delta + i beta
 *               (include/PyClass/RefractiveIndex.h:101-106)
 *   projection  float[num_energies][num_k][ny][nx]
 *   polarization complex float (re, im) [nz][ny][nx] per component
 */
#ifndef CYRSOXS_GB300_H
#define CYRSOXS_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define CYR_API __attribute__((visibility("default")))
#else
#define CYR_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define CYR_OK 0
#define CYR_ERR_ARGUMENT 1     /* invalid option or pointer */
#define CYR_ERR_UNSUPPORTED 2  /* option combination or size not implemented */
#define CYR_ERR_CUDA 3         /* CUDA runtime error (message in cyr_last_error) */
#define CYR_ERR_MEMORY 4       /* device memory could not be reserved */
#define CYR_ERR_NO_DEVICE 5    /* no CUDA device visible */
#define CYR_ERR_TIMEOUT 6      /* a bounded device wait gave up */

/*
 * Run options: the fields of the reference's InputData that the scattering
 * path reads (include/Input/InputData.h:160-232, setters :430-615).
 */
typedef struct cyr_options {
  uint32_t nx, ny, nz;         /* voxelDims[0..2] = X, Y, Z */
  uint32_t num_material;       /* NUM_MATERIAL (<= 32) */
  uint32_t num_energies;
  const float *energies;       /* eV, the order of the optical/projection arrays */
  float start_angle;           /* E-field rotation, degrees (setEAngles) */
  float end_angle;
  float increment_angle;
  float phys_size;             /* nm */
  uint32_t case_type;          /* 0 Default, 1 BeamDivergence, 2 GrazingIncidence */
  uint32_t num_k;              /* number of k vectors (1 for Default) */
  const float *k_vectors;      /* [num_k][3] unit vectors, as InputData stores them */
  float detector[3];           /* detectorCoordinates (GrazingIncidence) */
  uint32_t morphology_type;    /* 0 EulerAngles, 1 VectorMorphology */
  uint32_t ewald_interpolation;/* 0 NearestNeighbour, 1 Linear */
  uint32_t windowing;          /* 0 NoPadding, 1 Hanning (Algorithm 0 only) */
  uint32_t scatter_approach;   /* 0 Partial, 1 Full (numerically identical here) */
  uint32_t algorithm;          /* 0 CommunicationMinimizing, 1 MemoryMinimizing */
  uint32_t max_streams;        /* MaxStreams (accepted; the engine schedules itself) */
  uint32_t rot_mask;           /* RotMask */
  uint32_t reference_frame;    /* 1 Lab, 0 Material (the reference's bool values) */
  uint32_t strategy;           /* engine only (zero-initialised = auto): how the spectra are formed.
                                  1 PER_ENERGY: tensor-entry spectra per energy (per angle in the
                                  Material frame), as the reference's pipeline does;
                                  2 FIELDS: the 7 M + 1 energy-independent morphology fields are
                                  transformed once per request and combined per energy and angle
                                  at the Ewald sample points (exact by linearity of the FFT);
                                  0 AUTO: FIELDS when there are enough energies x angles to
                                  amortise it and its volumes fit the device, else PER_ENERGY. */
} cyr_options;

enum { CYR_STRATEGY_AUTO = 0, CYR_STRATEGY_PER_ENERGY = 1, CYR_STRATEGY_FIELDS = 2 };

/* Human-readable description of the last failure on this thread. */
CYR_API const char *cyr_last_error(void);

/* Library version string and the number of visible CUDA devices (or -1). */
CYR_API const char *cyr_version(void);
CYR_API int cyr_device_count(void);

/*
 * Full simulation from host buffers (host->device copy, all energies, k
 * vectors and E angles, device->host copy of the averaged projections).
 * Replaces cudaMain (include/cudaMain.h:53-60, src/cudaMain.cu:377-1035).
 */
CYR_API int cyr_cuda_main(const cyr_options *opt, const float *optical, const float *voxels, float *projection);

/*
 * Same contract for Algorithm 1 (MemoryMinimizing): replaces cudaMainStreams
 * (include/cudaMain.h:62-69, src/cudaMain.cu:1037-1667).  Windowing is not
 * applied, as in the reference.
 */
CYR_API int cyr_cuda_main_streams(const cyr_options *opt, const float *optical, const float *voxels, float *projection);

/*
 * Polarization of one energy (index energy_id) for an E rotation of eangle
 * RADIANS about the first k vector, before the FFT.  px/py/pz receive
 * complex float [nz][ny][nx] (re, im interleaved).  Replaces the debug
 * computePolarization (include/cudaMain.h:71-87, src/cudaMain.cu:1669-1738).
 */
CYR_API int cyr_compute_polarization(const cyr_options *opt, const float *optical, const float *voxels, float eangle,
                             uint32_t energy_id, float *px, float *py, float *pz);

/*
 * FP64 pipeline: the drop-in for the reference's -DDOUBLE_PRECISION build
 * (include/Datatypes.h:33-46: Real = double, Voxel::s1 a double4, cuFFT Z2Z),
 * with the same contract as cyr_cuda_main (include/cudaMain.h:53-60) on
 * double arrays: optical [E][M][4], voxels [M][Z][Y][X][4], projection
 * [E][K][Ny][Nx].  Every amplitude is computed in double (tensor, window, FFT,
 * DC replacement, intensity, interpolation, warps, angle mean); the discrete
 * decisions (NaN pixels, Ewald planes, warp taps) are made in float exactly as
 * the FP32 path makes them, so the NaN masks equal cyr_cuda_main's.  Axis
 * lengths must be 7-smooth (2^a 3^b 5^c 7^d).
 */
CYR_API int cyr_cuda_main_fp64(const cyr_options *opt, const double *optical, const double *voxels, double *projection);

/*
 * Device-resident FP64 pipeline: d_voxels holds float4 (voxels_fp64 = 0, the
 * FP32 path's own input, so the two can be compared on one morphology) or
 * double4 (voxels_fp64 = 1) voxels; d_projection receives doubles.
 * Asynchronous on `stream`; scratch is kept by the library (per device).
 */
CYR_API int cyr_simulate_device_fp64(const cyr_options *opt, const double *optical, const void *d_voxels,
                                     uint32_t voxels_fp64, double *d_projection, void *stream);

/*
 * FP64 polarization of one energy for an E rotation of eangle RADIANS:
 * replaces the FP64 build's computePolarization (include/cudaMain.h:71-87,
 * src/cudaMain.cu:1669-1738).  px/py/pz receive complex double [nz][ny][nx].
 */
CYR_API int cyr_compute_polarization_fp64(const cyr_options *opt, const double *optical, const double *voxels,
                                          double eangle, uint32_t energy_id, double *px, double *py, double *pz);

/*
 * Device-resident variant: voxels and projection are device pointers on the
 * current device; stream is a cudaStream_t (0 = legacy default stream).  The
 * call is asynchronous with respect to the host once it returns CYR_OK.
 * Scratch space is kept by the library between calls (per device).
 */
CYR_API int cyr_simulate_device(const cyr_options *opt, const float *optical, const void *d_voxels, float *d_projection,
                        void *stream);

/* Device bytes the engine needs for one request with these options. */
CYR_API int cyr_required_device_bytes(const cyr_options *opt, size_t *bytes);

/*
 * Shape of the engine's plan for these options: info[0] = spectrum volumes
 * per energy (5 or 6 tensor entries, 3 for the MATERIAL frame), info[1] =
 * z planes kept after the z FFT (nz when not pruned), info[2] = first kept
 * shifted plane, info[3] = 1 when the z axis is pruned, info[4] = E angles,
 * info[5] = k vectors, info[6] = 1 when the FIELDS strategy is chosen,
 * info[7] = packed field volumes, info[8] = energies per Ewald launch.
 */
CYR_API int cyr_plan_info(const cyr_options *opt, uint32_t *info, uint32_t n);

/*
 * Device-side consistency errors counted since the last request started on
 * this device (e.g. a detector pixel needed a z plane outside the kept
 * range).  Waits for the device; 0 means none.
 */
CYR_API int cyr_device_errors(uint32_t *count);

/*
 * The launch configurations the engine's autotuner chose on this device, one
 * line per shape ("kernel[shape]: choice time"), written into buf.
 */
CYR_API int cyr_tuning_report(char *buf, size_t len);

/* Releases the library's cached scratch space on the current device. */
CYR_API int cyr_release_scratch(void);

/*
 * Building blocks, exposed for parity tests of the individual stages.
 * All pointers are device pointers; calls are asynchronous on `stream`.
 *
 * cyr_fft3d_device: in-place forward unnormalised 3D DFT of `count`
 * consecutive complex [nz][ny][nx] volumes (cufftExecC2C FORWARD semantics,
 * include/cudaMain.h:184-190).  One volume may hold at most 2^32 - 1
 * elements (larger volumes are refused with CYR_ERR_ARGUMENT).
 */
CYR_API int cyr_fft3d_device(void *d_data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, void *stream);

/*
 * cyr_fft3d_device_static: the same transform as cyr_fft3d_device for callers
 * that cannot allocate device memory (code inside a memory pool or arena that
 * owns the device and forbids cudaMalloc/cudaFree, or latency-critical paths
 * that must not call allocating routines).  It calls no cudaMalloc, cudaFree
 * or allocating library routine: its twiddle tables live in a fixed 96 KiB
 * device array that is part of the library image and that every GPU loading
 * the library holds until the process exits.  Each axis may be at most 4096
 * long, and one volume at most 2^32 - 1 elements; larger sizes are rejected
 * with CYR_ERR_ARGUMENT.  The first call on a device resolves the array's
 * device address (cudaGetSymbolAddress) and sets the FFT kernel's
 * shared-memory limit, so make that first call before any stream capture.
 * Every call recomputes the tables in the array with a kernel on `stream`
 * (no host copy).  All calls share the array: calls whose work overlaps on
 * the GPU race.  This entry point has no counterpart in the reference.
 */
CYR_API int cyr_fft3d_device_static(void *d_data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count,
                                    void *stream);

/*
 * cyr_selftest_wait_limit: checks the bounded waits of the TMA column FFT pass.
 * It runs that kernel once on a 32 x 256 tile whose copies deliver fewer bytes
 * than the kernel's barrier expects, so every wait runs out; the kernel must
 * report it (*timed_out = 1), wait for the copies it issued, and leave the
 * context usable.  Returns CYR_ERR_TIMEOUT if the kernel could not confirm
 * within its wait limit that those copies landed.  Synchronises the device.
 * No counterpart in the reference.
 */
CYR_API int cyr_selftest_wait_limit(int *timed_out);

/*
 * cyr_warp_affine_device: bilinear affine warp of a float [height][width]
 * image with the semantics of nppiWarpAffine_32f_C1R + NPPI_INTER_LINEAR
 * (src/cudaMain.cu:91-121, :858, :943).  coeffs is the 2x3 matrix mapping
 * source to destination (host memory, row major); d_dst must already hold the
 * prefill value: pixels whose source falls outside the image keep it.
 */
CYR_API int cyr_warp_affine_device(const float *d_src, float *d_dst, int width, int height, const double *coeffs,
                           void *stream);

/*
 * Per-kernel timing.  Between cyr_profile_begin and cyr_profile_end every
 * kernel the engine launches is bracketed by a pair of CUDA events recorded
 * on its launch stream (no synchronisation is added).  cyr_profile_end waits
 * for the recorded events and returns, per kernel kind (cyr_stage_name), the
 * number of kernel launches, the number of timed calls (a call may launch a
 * matched pair of kernels of which one returns at entry) and their summed
 * duration in milliseconds.  Calls beyond max_launches are counted in
 * *dropped and not timed, and so are launches made while their stream is
 * being captured into a CUDA graph (the serving engine's graphs); replays of
 * a graph are not timed either.
 */
CYR_API int cyr_profile_begin(uint32_t max_launches);
CYR_API int cyr_profile_end(uint32_t *launches, uint32_t *calls, double *ms, uint32_t nstages, uint32_t *dropped);
CYR_API const char *cyr_stage_name(uint32_t stage);
CYR_API uint32_t cyr_num_stages(void);


/* ------------------------------------------------------------------------
 * Serving: continuous batching of simulation requests on the current device.
 * No counterpart in the reference, which runs one request per process call.
 *
 * A worker thread keeps up to `slots` requests in flight, each on its own
 * stream with its own scratch, so their work overlaps on the GPU.  Requests
 * are admitted in submission order as soon as a slot is free and their device
 * footprint (cyr_required_device_bytes, plus staging for host buffers) fits
 * in `hbm_budget` bytes next to the requests in flight (0: 85% of the free
 * memory at creation; a request larger than the budget runs alone).  Each
 * request computes exactly what cyr_cuda_main computes for it.  With
 * CYR_SERVER_GRAPHS a slot captures a CUDA graph of a request signature
 * (options and buffer pointers) the second time it runs it, and replays it
 * for later requests with the same signature.
 * ------------------------------------------------------------------------ */
typedef struct cyr_server cyr_server;
#define CYR_SERVER_GRAPHS 1u
/* With CYR_SERVER_GROUPS, queued requests that differ only in morphology,
 * energies and optical constants (FIELDS strategy, LAB frame, k along z,
 * device buffers, same shape, angles and options) are admitted together, up
 * to 16 at a time, and share one launch per kernel: the transform runs over
 * all their packed volumes at once, and the Ewald projection, rotation and
 * detector warp over all their energies.  Each request still computes
 * exactly what it computes alone. */
#define CYR_SERVER_GROUPS 2u

CYR_API int cyr_server_create(uint32_t slots, size_t hbm_budget, uint32_t flags, cyr_server **server);

/* Queues one request; options, energies, k vectors and optical constants are
 * copied.  device_buffers = 0: `voxels` [M][Z][Y][X] float4 and `projection`
 * [E][k][Ny][Nx] are host buffers (pinned memory lets the copies overlap other
 * requests); 1: device buffers.  They must stay valid until the request is
 * done.  The AUTO strategy is resolved here. */
CYR_API int cyr_server_submit(cyr_server *server, const cyr_options *opt, const float *optical, const void *voxels,
                              float *projection, uint32_t device_buffers, uint64_t *id);

/* done = 1 once the request has finished (its outputs are written). */
CYR_API int cyr_server_poll(cyr_server *server, uint64_t id, int *done);

/* Blocks until the request has finished and returns its status; latency_s
 * (submit to completion) and queue_s (submit to admission) may be null.  The
 * id is forgotten afterwards. */
CYR_API int cyr_server_wait(cyr_server *server, uint64_t id, double *latency_s, double *queue_s);

CYR_API int cyr_server_stats(cyr_server *server, uint64_t *completed, uint64_t *failed, uint64_t *graph_replays,
                             uint64_t *graph_captures);

/* Number of grouped launches (CYR_SERVER_GROUPS) and the requests they served. */
CYR_API int cyr_server_group_stats(cyr_server *server, uint64_t *group_runs, uint64_t *grouped_requests);

/* Finishes the queued requests, then frees the slots. */
CYR_API int cyr_server_destroy(cyr_server *server);

#ifdef __cplusplus
}
#endif

#endif /* CYRSOXS_GB300_H */
