/*
 * valomc_gb300.h -- C ABI of the GB300 photon-propagation engine.
 *
 * Drop-in for the hot path of ValoMC: everything from MC3D::MonteCarlo's parallel region
 * through the reduction and normalisation (cpp/3d/MC3D.hpp:1641-1822, cpp/2d/MC2D.hpp:1514-1707)
 * plus the setup that feeds it (ErrorChecks :460-571, Init :576-738).  The callers it
 * serves are the MEX gateways (cpp/3d/MC3Dmex.cpp:98-253, cpp/2d/MC2Dmex.cpp:98-252) and
 * the external executables (cpp/3d/MC3D.cpp:34-94, cpp/2d/MC2D.cpp:38-122).
 *
 * Conventions
 *   - Plain C: pointers, sizes, status codes.  No exception crosses this boundary.
 *   - Index and coordinate arrays use the reference's Array<T> layout
 *     (cpp/3d/Array.hpp:58-69): column-major, row index fastest, H(el, c) = H[el + Ne*c],
 *     0-based, int64 indices and double values -- exactly what MC3Dmex receives.
 *   - Inputs are borrowed for the duration of the call; outputs are caller-allocated.
 *   - Every array carries its own row count so that ErrorChecks' size checks keep
 *     their codes and order.
 *   - Device memory is owned by the library (per call, or by a resident mesh handle).
 *   - vmc_run and vmc_run_batch each run on a non-blocking stream of their own, so calls
 *     from several host threads overlap on the GPU; a resident mesh may be shared by
 *     concurrent calls (they only read it).  vmc_run_noalloc also runs on a stream of its
 *     own, but its calls share one scratch array and must not overlap (below).
 */
#ifndef VALOMC_GB300_H
#define VALOMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VMC_ABI_VERSION 1

/* ---------------------------------------------------------------------------------- */
/* Status codes.  1..16 are 1 + the reference's mcerror values (cpp/Errors.hpp:4-21),   */
/* in the same order; the rest are conditions the reference has no code for.           */
/* ---------------------------------------------------------------------------------- */
enum vmc_status {
  VMC_OK = 0,
  VMC_NO_LIGHTSOURCE = 1,
  VMC_SIZE_MISMATCH_G = 2,
  VMC_SIZE_MISMATCH_MUA = 3,
  VMC_SIZE_MISMATCH_MUS = 4,
  VMC_SIZE_MISMATCH_N = 5,
  VMC_SIZE_MISMATCH_BCN = 6,
  VMC_MISSING_BCN = 7,
  VMC_SIZE_MISMATCH_BCTYPE = 8,
  VMC_SIZE_MISMATCH_LIGHT_DIRECTION = 9,
  VMC_SIZE_MISMATCH_LIGHT_DIRECTION_TYPE = 10,
  VMC_INCONSISTENT_H = 11,
  VMC_INCONSISTENT_BH = 12,
  VMC_INCONSISTENT_MESH = 13,
  VMC_INCONSISTENT_MESH_DUPLICATE_NEIGHBORS = 14,
  VMC_NO_GAUSSIAN_SIGMA = 15,
  VMC_MISSING_BOUNDARY = 16,
  VMC_ERR_INVALID_ARGUMENT = 32,  /* null pointer, bad dim, bad option */
  VMC_ERR_CUDA = 33,              /* a CUDA runtime call failed; see vmc_last_error() */
  VMC_ERR_NO_DEVICE = 34,         /* no CUDA device, or not an sm_103 part */
  VMC_ERR_OUT_OF_MEMORY = 35,
  VMC_ERR_CANCELLED = 36,         /* progress callback returned 0 or *cancel was set */
  VMC_ERR_TIMEOUT = 37,           /* options.timeout_s elapsed; the kernel was stopped */
  VMC_ERR_TAPE = 38,              /* replay tape shorter than a photon's draws */
  VMC_ERR_ADMISSION = 39,         /* serving: request larger than the memory budget */
  VMC_ERR_NOT_FOUND = 40,         /* serving: unknown request or mesh id */
  VMC_ERR_SIZE_LIMIT = 41         /* a size beyond a stated maximum */
};

/* arithmetic form of the photon walk */
enum vmc_precision {
  VMC_FP64 = 0, /* plain form: the reference's FP64 arithmetic and Moller-Trumbore face test */
  VMC_FP32 = 1  /* tracking form: FP32 position/direction/weight, barycentric (plane)
                   exit test robust to rounding, FP64 accumulators */
};

/* uniform source */
enum vmc_rng {
  VMC_RNG_PHILOX = 0, /* Philox4x32-10 per photon: key = seed, counter = (photon, block, stream) */
  VMC_RNG_TAPE = 1    /* photon p consumes tape[tape_off[p] .. tape_off[p+1]) (trajectory replay) */
};

/* trace codes written by the replay trace: deposits are element indices >= 0, exits are
 * -1 - ib, and a photon's last entry is one of these when it did not exit */
#define VMC_EV_ROULETTE (INT64_MIN + 1)
#define VMC_EV_LOST (INT64_MIN + 2)
#define VMC_EV_CAPPED (INT64_MIN + 3)
#define VMC_EV_TAPE_END (INT64_MIN + 4)
#define VMC_EV_TRUNCATED (INT64_MIN + 5)

/* progress callback: percent of photons started; return 0 to abort (the reference's
 * progress(double) -> bool, cpp/3d/MC3D.hpp:1688) */
typedef int (*vmc_progress_fn)(double percent, void *user);

/* One problem: the arrays MC3Dmex / MC2Dmex receive, same meaning and order
 * (cpp/3d/MC3Dmex.cpp:122-139, cpp/2d/MC2Dmex.cpp:122-140).  n_* are row counts. */
typedef struct vmc_input {
  int32_t dim;                       /* 3 (tetrahedra, MC3D) or 2 (triangles, MC2D) */
  int32_t seed_given;                /* rndseed[1] (cpp/3d/MC3Dmex.cpp:167-176): 0 = clock seed */
  int64_t Ne, Nb, Nr;                /* rows of H, BH, r */
  const int64_t *H;                  /* [Ne x (dim+1)] element nodes */
  const int64_t *HN; int64_t n_HN;   /* optional neighbourhood [n_HN x (dim+1)]; built when n_HN != Ne */
  const int64_t *BH;                 /* [Nb x dim] boundary element nodes */
  const double *r;                   /* [Nr x dim] node coordinates */
  const char *BCType; int64_t n_BCType;
  const double *BCIntensity; int64_t n_BCIntensity;            /* 0 rows: all 1 */
  const char *BCLightDirectionType; int64_t n_BCLightDirectionType; /* 0 rows: all 'n' */
  const double *BCLNormal; int64_t n_BCLNormal;                /* [n x dim] */
  const double *BCn; int64_t n_BCn;
  const double *mua; int64_t n_mua;
  const double *mus; int64_t n_mus;
  const double *g; int64_t n_g;
  const double *n; int64_t n_n;
  double f;                          /* modulation frequency [Hz]; 0 = continuous wave */
  double phase0;                     /* initial phase; negative values are wrapped to [0, 2 pi) */
  int64_t Nphoton;
  const double *GaussianSigma; int64_t n_GaussianSigma;        /* 2D 'g' sources */
  uint64_t seed;                     /* rndseed[0] */
} vmc_input;

/* caller-allocated results, laid out like the MEX outputs (real and imaginary parts) */
typedef struct vmc_output {
  double *ER, *EI;     /* [Ne] element fluence (vsol) */
  double *EBR, *EBI;   /* [Nb] boundary exitance (bsol) */
  double *DEBR, *DEBI; /* [Nb] direction-weighted exitance (ebsol; zero in 3D); may be NULL */
  int64_t *HN;         /* optional [Ne x (dim+1)] neighbourhood used (the MEX 6th output) */
} vmc_output;

typedef struct vmc_options {
  int32_t precision;        /* enum vmc_precision */
  int32_t rng;              /* enum vmc_rng */
  int32_t device;           /* CUDA device ordinal */
  int32_t block_size;       /* threads per block; 0 = tuned default */
  int32_t blocks_per_sm;    /* 0 = as many as fit */
  int32_t fetch_chunk;      /* photons a warp reserves per counter update; 0 = default */
  int64_t max_steps;        /* per-photon element-step cap (capped photons are reported); 0 = 10^7,
                               at most 2^31 - 1 */
  double timeout_s;         /* 0 = none */
  uint32_t stream_id;       /* Philox counter word 3: independent streams for the same seed */
  int32_t normalize;        /* 1 (default when options == NULL): apply MonteCarlo's normalisation */
  vmc_progress_fn progress; void *progress_user;
  const volatile int32_t *cancel;  /* polled by the host thread while the GPU runs */
  /* replay (rng == VMC_RNG_TAPE) */
  const uint32_t *tape; const int64_t *tape_off; int64_t tape_photons;
  /* optional per-photon trace of photons [0, trace_photons) */
  int64_t *trace; int64_t *trace_len; int64_t trace_stride; int64_t trace_photons;
  /* photon index offset: this call simulates photons [photon_offset, photon_offset+Nphoton)
   * of the seed's stream (disjoint replicas, resumable runs) */
  int64_t photon_offset;
  /* 1: record the launch (control-block reset + persistent kernel) as a CUDA graph and run
   * the instantiated graph; repeated launches of the same shape update and reuse it */
  int32_t use_graph;
  /* Shared-memory staging of the FP64 accumulators, per CTA, added to global memory once
   * when the CTA ends.
   * > 0: a hashed table of this many element slots (rounded up to a power of 2, at most
   *      4096) for the element fluence (FP32 tetrahedral walk, continuous wave, single job);
   *   0: (default) the whole accumulator set, 2 Ne + 4 Nb doubles, when the launch runs one
   *      job, the set fits in 32 KB and the shared memory costs no resident CTA;
   * < 0: no staging: every addition is a global reduction. */
  int32_t stage_slots;
  /* a warp relaunches its idle lanes once at least this many are idle, or on every 8th
   * loop iteration, so that short walks launch their photons together; 0 = default */
  int32_t refill_lanes;
} vmc_options;

typedef struct vmc_stats {
  int64_t photons_requested;
  int64_t photons_done;     /* photons whose walk ended */
  int64_t loss;             /* photons without an exit face or reverse face (the reference's 'loss') */
  int64_t capped;           /* photons stopped by max_steps */
  int64_t steps;            /* element steps (one WhichFace + move + score each) */
  int64_t scatters;
  int64_t roulette_kills;
  uint64_t seed_used;
  double seconds_setup;     /* host ErrorChecks/Init work and uploads */
  double seconds_kernel;    /* photon-pool kernel, CUDA events */
  double seconds_total;     /* whole call */
  double ledger[8];         /* launched, absorbed, exited, roulette_kill, roulette_gain, lost (weights) */
  int32_t grid_blocks, block_size;
  int32_t status_detail;    /* device error flags (tape end, bad index) */
  int32_t reserved;
  int64_t bytes_h2d;        /* host-to-device bytes this call copied */
  int64_t bytes_d2h;        /* device-to-host bytes this call copied */
} vmc_stats;

/* ---------------------------------------------------------------------------------- */
/* Entry points                                                                         */
/* ---------------------------------------------------------------------------------- */

/* ABI version and the reference's error strings for codes 1..16 (cpp/Errors.hpp:24-58). */
int vmc_abi_version(void);
const char *vmc_status_string(int status);
/* text of the last CUDA / internal error on this thread */
const char *vmc_last_error(void);

/* Fills options with defaults (FP32 form, Philox, device 0, normalised output). */
void vmc_default_options(vmc_options *opt);

/* One simulation: ErrorChecks + Init + MonteCarlo on the GPU + normalisation.
 * Replaces mexFunction's compute core (cpp/3d/MC3Dmex.cpp:178-236 and
 * cpp/2d/MC2Dmex.cpp:176-235) and the executables' ErrorChecks/Init/MonteCarlo
 * sequence (cpp/3d/MC3D.cpp:65-77, cpp/2d/MC2D.cpp:89-104). */
int vmc_run(const vmc_input *in, const vmc_options *opt, vmc_output *out, vmc_stats *stats);

/* Setup only: ErrorChecks and BuildNeighbourhoods (cpp/3d/MC3D.hpp:460-571, :835-871).
 * Writes HN [Ne x (dim+1)] (boundary faces -1 - ib; a 3D face with no neighbour stays
 * INT64_MAX as in the reference).  Used by createBH-style tooling and tests. */
int vmc_build_neighbourhood(const vmc_input *in, int64_t *HN_out);

/* Resident meshes: geometry uploaded once and reused by many jobs (batching, serving). */
typedef struct vmc_mesh vmc_mesh;
int vmc_mesh_create(const vmc_input *geometry, int32_t precision, int32_t device, vmc_mesh **out);
int vmc_mesh_destroy(vmc_mesh *mesh);
int64_t vmc_mesh_device_bytes(const vmc_mesh *mesh);

/* Many problems in one persistent launch.  jobs[j] holds the optics, boundary conditions,
 * f, phase0, Nphoton and seed of job j (geometry pointers may be NULL: meshes[j] is used);
 * outs[j] receives job j's results.  stats (optional) gets the totals, job_stats
 * (optional, njobs entries) the per-job counters. */
int vmc_run_batch(vmc_mesh *const *meshes, const vmc_input *jobs, int32_t njobs,
                  const vmc_options *opt, vmc_output *outs, vmc_stats *stats, vmc_stats *job_stats);

/* Autotuner: times short runs of a problem over block sizes x blocks per SM x fetch
 * chunks, then, on the fastest shape, the idle lanes a warp waits for before relaunching
 * them (refill_lanes), and writes the result into opt (precision and rng are kept). */
int vmc_autotune(vmc_mesh *const *meshes, const vmc_input *jobs, int32_t njobs, vmc_options *opt,
                 double budget_s);

/* Serving: resident meshes, requests admitted by device-memory footprint, continuous
 * batching of request slots into short persistent launches. */
typedef struct vmc_server vmc_server;
enum vmc_slicing {
  VMC_SLICE_DEFAULT = 0,         /* the server's choice: shortest remaining first */
  VMC_SLICE_EQUAL = 1,           /* water-filling: requests below an equal share get all they
                                    have left, the others share the rest equally */
  VMC_SLICE_SHORTEST_FIRST = 2   /* every open request a floor of 1/4 of an equal share, the
                                    rest to the requests with the fewest photons left first */
};
typedef struct vmc_server_config {
  int32_t device;
  int32_t precision;
  int32_t max_slots;          /* requests simulated concurrently */
  int32_t use_graph;          /* run each epoch's launches as an updated CUDA graph */
  int64_t memory_budget;      /* bytes of per-request device state admitted at once; clamped
                                 to the device's free memory (less 256 MiB) at creation */
  int64_t epoch_photons;      /* photons per launch across all slots; 0 = by load: 50 ms of
                                 work at the measured rate while the backlog is small, up to
                                 the backlog and epoch_max_ms of work as it grows */
  int32_t block_size, blocks_per_sm;
  int32_t slicing;            /* enum vmc_slicing: how an epoch's photons are shared among requests */
  int32_t epoch_max_ms;       /* cap of an epoch sized by load, in ms of work at the measured
                                 rate (>= 50); 0 = 500.  Larger epochs pay the end-of-launch
                                 drain less often (capacity); smaller ones let new requests
                                 in sooner (latency) */
} vmc_server_config;
int vmc_server_create(const vmc_server_config *cfg, vmc_server **out);
int vmc_server_add_mesh(vmc_server *s, vmc_mesh *mesh, int32_t *mesh_id);   /* server borrows mesh */
/* copies the job's arrays; returns a request id (> 0) in *req_id */
int vmc_server_submit(vmc_server *s, int32_t mesh_id, const vmc_input *job, int64_t *req_id);
/* 1 = finished (results copied to out), 0 = pending, < 0 = -status */
int vmc_server_poll(vmc_server *s, int64_t req_id, vmc_output *out, vmc_stats *stats);
int vmc_server_wait(vmc_server *s, int64_t req_id, vmc_output *out, vmc_stats *stats, double timeout_s);
int vmc_server_destroy(vmc_server *s);

/* ---------------------------------------------------------------------------------- */
/* Allocation-free run.  No counterpart in the reference.                               */
/*                                                                                      */
/* For callers that cannot let a library call cudaMalloc: hosts whose device memory is   */
/* owned end to end by their own allocator (a framework's caching allocator, or a pool  */
/* a serving process reserved up front), where a library-side cudaMalloc/cudaFree would */
/* synchronise the device and take memory outside their accounting.  The caller passes  */
/* the job's device arrays in buffers it owns (below) and receives host outputs; the    */
/* kernel's scratch (launch control block, job table, event counters, emitting-face     */
/* records) lives in one file-scope device array of VMC_NOALLOC_SCRATCH_BYTES that every */
/* GPU which loads the library holds until the process exits.                           */
/*                                                                                      */
/* - The geometry comes from a resident mesh created beforehand (vmc_mesh_create).       */
/* - One job per call, Philox streams only, at most VMC_NOALLOC_MAX_SOURCES emitting     */
/*   faces; larger problems are refused with VMC_ERR_SIZE_LIMIT and a message.           */
/* - The first call on a device looks up the scratch array's device address with that    */
/*   device current; make that first call before any stream capture.                     */
/* - Every call reuses the same scratch and clears what must start at zero; calls that   */
/*   overlap on the GPU (other threads, other streams) race on it: serialise them.       */
/* - It calls no cudaMalloc, cudaFree or other allocating device routine.                */
/* - It runs on a non-blocking stream of its own and returns when its work is done; it   */
/*   does not wait for the caller's streams, so no work in flight may still use `dev`.   */
/* - `dev` must be device memory of options.device, the device the mesh lives on; other  */
/*   pointers are refused (VMC_ERR_INVALID_ARGUMENT).                                    */
/* - It polls no progress callback, cancel flag or timeout (options that set one are     */
/*   refused); use_graph and stage_slots are not used.                                   */
/* - The cached scratch address belongs to the device's primary context: after           */
/*   cudaDeviceReset on a device, do not call it on that device again.                   */
#define VMC_NOALLOC_SCRATCH_BYTES (256 * 1024)
#define VMC_NOALLOC_MAX_SOURCES 512

typedef struct vmc_noalloc_buffers {
  void *optics;     /* [Ne x 4] rows (mua, mus, g, n): float for VMC_FP32, double for VMC_FP64 */
  uint8_t *bctype;  /* [Nb] boundary condition codes */
  double *bcn;      /* [Nb] exterior refractive indices */
  double *acc;      /* [2 Ne + 4 Nb] raw accumulators ER, EI, EBR, EBI, DEBR, DEBI */
} vmc_noalloc_buffers;

/* The job's optics / boundary arrays come from `job` (geometry pointers are ignored: the
 * mesh is used), are copied into `dev`, and the normalised results are written to the
 * host arrays of `out`, as vmc_run does. */
int vmc_run_noalloc(vmc_mesh *mesh, const vmc_input *job, const vmc_options *opt, const vmc_noalloc_buffers *dev,
                    vmc_output *out, vmc_stats *stats);

/* Micro-benchmarks for the roofline denominators: random 32-byte-sector gathers over a
 * buffer of 'bytes' (dependent chains, like the element walk), and an FP64 FMA loop. */
int vmc_bench_gather(int32_t device, int64_t bytes, double seconds, double *gbs_out);
int vmc_bench_fp64(int32_t device, double seconds, double *tflops_out);

#ifdef __cplusplus
}
#endif
#endif
