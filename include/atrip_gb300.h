/*
 * atrip_gb300 -- C ABI of the GB300 CCSD(T) triples engine.
 *
 * This is the boundary under atrip's public C++ API (atrip::Atrip::Input /
 * Atrip::run / Atrip::Output, src/atrip/Atrip.hpp:41-140).  The header-only
 * C++ drop-in in include/atrip/Atrip.hpp calls these entry points; a host in
 * any language can bind them directly (plain pointers, sizes, status codes,
 * no CUDA or torch types in any signature).
 *
 * One context owns one GPU's worth of state: the HBM-resident operand
 * tensors in kernel-friendly layouts, the tuple work queue and the per-tuple
 * energy array.  It replaces atrip's per-rank state (the static members of
 * struct Atrip, src/atrip/Atrip.hpp:43-63), its SliceUnions
 * (src/atrip/Atrip.cxx:277-362) and its tuple distribution
 * (src/atrip/Tuples.hpp:49-52).  Contexts are independent; one context must
 * not be used from two host threads at once.
 *
 * All input arrays are FP64 and column-major (first index fastest), i.e.
 * exactly what CTF::Tensor::read_all returns for atrip's inputs.
 *
 * Every entry point returns ATRIP_OK (0) or a status below; the text of the
 * last error on the calling thread is available from atrip_gpu_last_error().
 */
#ifndef ATRIP_GB300_H
#define ATRIP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  atrip throws const char* / std::string on failure
 * (src/atrip/Acc.hpp:16-41, src/atrip/CUDA.hpp:27-38); the C++ drop-in turns
 * a non-zero status into a thrown std::string with atrip_gpu_last_error(). */
enum atrip_status {
  ATRIP_OK = 0,
  ATRIP_ERR_ARGUMENT = 1,      /* bad pointer, size, tensor id or option   */
  ATRIP_ERR_CUDA = 2,          /* a CUDA runtime call failed               */
  ATRIP_ERR_OUT_OF_MEMORY = 3, /* device allocation failed                 */
  ATRIP_ERR_STATE = 4,         /* missing input, or call out of order      */
  ATRIP_ERR_TIMEOUT = 5,       /* a device-side bounded wait gave up       */
  ATRIP_ERR_UNSUPPORTED = 6,   /* size or form this build does not support */
  ATRIP_ERR_NO_DEVICE = 7      /* no usable sm_103 device                  */
};

/* Input tensors, named after atrip's Input::with_* builders
 * (src/atrip/Atrip.hpp:72-107).  Shapes (column-major):
 *   EPSI  (No)            EPSA  (Nv)           TAI   (Nv,No)
 *   TABIJ (Nv,Nv,No,No)   VABIJ (Nv,Nv,No,No)  VIJKA (No,No,No,Nv)
 *   VABCI (Nv,Nv,Nv,No)   JIJKA (No,No,No,Nv)  JABCI (Nv,Nv,Nv,No)      */
enum atrip_tensor {
  ATRIP_EPSI = 0,
  ATRIP_EPSA = 1,
  ATRIP_TAI = 2,
  ATRIP_TABIJ = 3,
  ATRIP_VABIJ = 4,
  ATRIP_VIJKA = 5,
  ATRIP_VABCI = 6,
  ATRIP_JIJKA = 7,
  ATRIP_JABCI = 8,
  ATRIP_N_TENSORS = 9
};

/* Arithmetic form of the contractions. */
enum atrip_form {
  ATRIP_FORM_FP64 = 0,       /* FP64 throughout                               */
  ATRIP_FORM_SPLIT_BF16 = 1, /* operands cut into BF16 slices, tensor cores,  */
                             /* FP32 accumulation, FP64 recombination         */
  ATRIP_FORM_AUTO = 2,       /* split-BF16 for real inputs (3 slices unless  */
                             /* given), FP64 for complex                      */
  ATRIP_FORM_SPLIT_F16 = 3   /* 2 FP16 slices of 11-bit digits (22 bits per  */
                             /* operand, the MMAs of 2 BF16 slices); level 0  */
                             /* FP32-rounded; needs No <= 64 and              */
                             /* 2 (Nv + No) < 2048                            */
};

/* Field of the inputs (atrip's Atrip::run<double> / run<Complex>,
 * src/atrip/Atrip.cxx:1135-1136). */
enum atrip_field {
  ATRIP_FIELD_REAL = 0,    /* FP64 elements                                  */
  ATRIP_FIELD_COMPLEX = 1  /* std::complex<double>: interleaved (re, im) FP64 */
};

typedef struct atrip_gpu_context atrip_gpu_context;

typedef struct {
  int32_t no;     /* occupied orbitals, 1 <= no <= 64   */
  int32_t nv;     /* virtual orbitals,  1 <= nv <= 1023 */
  int32_t device; /* CUDA device ordinal                */
  int32_t field;  /* enum atrip_field (0 = real)        */
} atrip_dims;

/* Options of one run; mirrors the Input attributes that change results or
 * the tuple range (src/atrip/Atrip.hpp:113-131).  Zero-initialise and set
 * what you need. */
typedef struct {
  int32_t form;            /* enum atrip_form                                  */
  int32_t slices;          /* split forms: slices per operand, BF16 2..4       */
                           /* (0: 3), FP16 2 (0: 2)                            */
  int32_t ijkabc;          /* Input::ijkabc: negate T1, skip final negation    */
  int32_t use_j;           /* 1: (cT) with JIJKA/JABCI when both uploaded      */
  int64_t first_iteration; /* resume cursor (checkpoint Iteration)             */
  int64_t max_iterations;  /* Input::max_iterations: 0 = all; else tuples      */
                           /* first_iteration .. max_iterations inclusive      */
  double start_energy;     /* checkpoint Energy (physical sign), added back    */
  void *stream;            /* cudaStream_t to run on, NULL = context stream    */
} atrip_run_options;

typedef struct {
  double energy;         /* Output::energy    (src/atrip/Atrip.hpp:134-137)   */
  double ct_energy;      /* Output::ct_energy                                 */
  int64_t tuples_done;   /* tuples processed in this run                      */
  int64_t next_iteration;/* cursor after the run (for checkpoints)            */
  double device_ms;      /* device time of the tuple loop (CUDA events)       */
  int32_t form_used;     /* enum atrip_form actually run                      */
  int32_t slices_used;   /* split form: slices per operand                    */
  int64_t kernel_launches; /* kernels this library launched in the run        */
} atrip_result;

/* Number of CUDA devices this process sees (0 without a driver or GPU).
 * Ranks of a multi-process run pick theirs from it (one GPU per rank, the
 * device assignment atrip's ranks get from their node-local rank). */
int atrip_gpu_device_count(int32_t *count);

/* Create a context on dims->device.  Replaces the per-rank device setup of
 * Atrip::run (src/atrip/Atrip.cxx:78-171) and the tuple list
 * (src/atrip/Tuples.cxx:89-134, built once on the host, kept on device). */
int atrip_gpu_create(const atrip_dims *dims, atrip_gpu_context **out);

/* Upload one input tensor from host memory (pageable or pinned), n_elements
 * values in column-major order (FP64, or (re, im) FP64 pairs for a complex
 * context: n_elements counts complex values).  The device copy is kept in
 * the engine's own layout.  Replaces read_all + the SliceUnion constructors
 * (src/atrip/Atrip.cxx:176-215, 277-362; src/atrip/Unions.hpp:77-278).     */
int atrip_gpu_upload(atrip_gpu_context *ctx, int32_t tensor, const double *host_colmajor,
                     int64_t n_elements);

/* Same from device memory (a column-major FP64 array already in HBM). */
int atrip_gpu_upload_device(atrip_gpu_context *ctx, int32_t tensor,
                            const double *device_colmajor, int64_t n_elements);

/* Drop an uploaded tensor (atrip's Input::delete_Vppph,
 * src/atrip/Atrip.cxx:310, frees the caller's V_pphp after slicing). */
int atrip_gpu_release(atrip_gpu_context *ctx, int32_t tensor);

/* Run the triples loop over the tuple range selected by opts and reduce the
 * energies.  Replaces the per-tuple loop and the final reduction of
 * Atrip::run (src/atrip/Atrip.cxx:686-1111): doubles_contribution,
 * singles_contribution and get_energy_{same,distinct}
 * (src/atrip/Equations.cxx:101-238, 387-426, 455-728). Blocks until done. */
int atrip_gpu_run(atrip_gpu_context *ctx, const atrip_run_options *opts, atrip_result *out);

/* Launch parameters chosen by the autotuner (atrip_gb300/autotune.py);
 * a zero field keeps the built-in choice.  No counterpart in the reference,
 * whose only tuning knob for this loop is the tuple distribution.          */
typedef struct {
  int32_t fp64_ctas_per_sm; /* FP64 form: resident CTAs per SM (0 = occupancy max) */
  int32_t fp64_tile_rows;   /* FP64 form: (p,q) rows per register tile, 32 or 64    */
  int32_t tuples_per_claim; /* FP64 form: tuples a CTA takes per queue access       */
  int32_t split_stages;     /* split form: operand ring depth, 2..6 (0 = all fit)   */
  int32_t split_ctas;       /* split form: persistent CTAs, <= SMs (0 = one per SM) */
  int32_t fp64_min_blocks;  /* FP64 form: 2 = kernel built for 2 CTAs/SM (<= 128   */
                            /* registers), 0 = register budget left to the compiler */
  int32_t split_w_global;   /* split form: 1 = energy warps read W from L2 even   */
                            /* when its FP64 copy fits in shared memory (No <= 24), */
                            /* leaving that memory to a deeper operand ring        */
  int32_t tuple_block;      /* processing order of the run's tuples: 0/1 = list    */
                            /* order; L >= 2 = grouped by (a/L, b/L, c/L) blocks,  */
                            /* so the tuples in flight share their a, b, c slabs   */
                            /* in L2 (results are unchanged: per-tuple energies    */
                            /* stay indexed by list position)                      */
  int32_t split_variant;    /* split form kernel: 0/1 = M tiles of (p,q) rows;     */
                            /* 2 = transposed (the S slices of V stacked as the    */
                            /* M rows, up to 256 (p,q) pairs as N) where S No <=   */
                            /* 128 and 2 (Nv + No) <= 1024, else variant 1;        */
                            /* 3 = 2 with one stack load per K chunk shared by the */
                            /* S slice units (No % 8 == 0), else variant 2          */
  int32_t split_prefetch;   /* split form: 1 = prefetch the next part's T / V_hhhp  */
                            /* slab tiles into L2 while the current part streams   */
  int32_t split_wait_kcycles; /* split form: limit of every device-side bounded   */
                            /* wait in thousands of SM cycles (0 = ~2 s); a wait   */
                            /* that runs out ends the launch, the run returns      */
                            /* ATRIP_ERR_TIMEOUT and the context stays usable      */
  int32_t split_test_unpublished; /* test of that path: 1 = the kernel's producer */
                            /* publishes no tuple, so every other role's first    */
                            /* wait runs out (no copy or MMA is issued); 0 = off   */
  int32_t split_profile;    /* split form: 1 = run the kernel built with per-role  */
                            /* cycle counters (2 slices, transposed kernel only;   */
                            /* same results), read by atrip_gpu_split_profile      */
} atrip_tuning;

/* Set / read the context's launch parameters (kept until changed). */
int atrip_gpu_set_tuning(atrip_gpu_context *ctx, const atrip_tuning *tuning);
int atrip_gpu_get_tuning(const atrip_gpu_context *ctx, atrip_tuning *tuning);

/* The compensated sums behind the last run's result: sums[0] + sums[1] is
 * the sum of its per-tuple energies (sums[1] the Neumaier compensation of
 * sums[0]), sums[2] + sums[3] likewise for the (cT) energies; no sign and
 * no checkpoint energy applied.  Processes that each run one contiguous
 * share of the tuple list merge these pairs into the total exactly as
 * atrip's final MPI_Reduce of the local energies does
 * (src/atrip/Atrip.cxx:1094-1107), without the rounding of one double per
 * process.                                                                 */
int atrip_gpu_last_sums(const atrip_gpu_context *ctx, double *sums);

/* Role profile of the last split-form run made with tuning split_profile = 1:
 * SM cycles summed over the CTAs (clock64 on each role's leading thread),
 *   [0] producer total      [1] producer waiting for a free ring stage
 *   [2] producer waiting for a free tuple slot
 *   [3] MMA issuer total    [4] ... waiting for a tuple   [5] ... for a free
 *       accumulator          [6] ... for a filled ring stage
 *   [7] epilogue total      [8] ... waiting for a tuple   [9] ... for a free
 *       W buffer             [10] ... for a finished accumulator
 *   [11] energy total       [12] ... waiting for a tuple  [13] ... for the
 *       tuple's W            [14] ... converting W to FP64
 *   [16] ring stages consumed  [17] tuples  [18] CTAs   (others 0)
 * The reference's closest facility is its per-section Timings
 * (src/atrip/Atrip.hpp:47); this one times the device roles instead. */
#define ATRIP_SPLIT_PROFILE_COUNTERS 20
int atrip_gpu_split_profile(const atrip_gpu_context *ctx, uint64_t *counters, int32_t n);

/* Per-tuple energies of the last run, tuple-list positions t0 .. t0+n-1
 * (the sign atrip accumulates before its final negation). ect may be NULL. */
int atrip_gpu_tuple_energies(atrip_gpu_context *ctx, int64_t t0, int64_t n, double *e,
                             double *ect);

/* Number of tuples for nv (src/atrip/Tuples.cxx:93) and the (a,b,c) of list
 * position t (src/atrip/Tuples.cxx:122-134).  No context needed.           */
int64_t atrip_gpu_n_tuples(int32_t nv);
int atrip_gpu_tuple_at(int32_t nv, int64_t t, int32_t *a, int32_t *b, int32_t *c);

/* Destroy a context and free its device memory. */
int atrip_gpu_destroy(atrip_gpu_context *ctx);

/* Text of the last failure on this host thread ("" if none). */
const char *atrip_gpu_last_error(void);

/* Library version string. */
const char *atrip_gpu_version(void);

/* Measured FP64 (DFMA) and FP32 (FFMA) throughput of the device in TFLOP/s,
 * from a short on-device timing loop (used as roofline denominators). */
int atrip_gpu_measure_peaks(int32_t device, double *fp64_tflops, double *fp32_tflops);

/* ---------------------------------------------------------------------
 * Batching form: many independent systems in one run.
 *
 * The reference runs one system per Atrip::run (src/atrip/Atrip.cxx:78-1111);
 * a batch replaces a host loop of such calls over small molecules.  Both
 * forms run every system's tuples in ONE persistent launch over a shared
 * device work queue (the split form keeps each system's tensor maps in a
 * device table; where one shared-memory layout cannot serve all systems it
 * falls back to one launch per system).  The sequence is captured into a
 * CUDA graph on the first run and replayed by later runs with the same
 * form, slice count and range.
 *
 * atrip_gpu_batch_create: systems[0..n-1] are contexts on one device with
 * No <= 32; the batch keeps the pointers (destroy the batch before any of
 * them).
 * atrip_gpu_batch_run: opts as for atrip_gpu_run, applied to every system
 * (start_energy must be 0); results[s] belongs to systems[s], its
 * device_ms and kernel_launches cover the whole batch.  Afterwards
 * atrip_gpu_tuple_energies works on each context as after atrip_gpu_run.
 * atrip_gpu_batch_plan: the launch order (cost-descending, stable) the
 * batch gives systems with these sizes; host-only, needs no device.       */
typedef struct atrip_gpu_batch atrip_gpu_batch;

int atrip_gpu_batch_create(atrip_gpu_context *const *systems, int32_t n, atrip_gpu_batch **out);
int atrip_gpu_batch_run(atrip_gpu_batch *batch, const atrip_run_options *opts,
                        atrip_result *results);
int atrip_gpu_batch_destroy(atrip_gpu_batch *batch);
int atrip_gpu_batch_plan(const int32_t *no, const int32_t *nv, int32_t n, int32_t *order);
/* FP64 launch parameters of the batch kernel (fp64_ctas_per_sm,
 * fp64_min_blocks, tuples_per_claim); the row tile is each context's own
 * fp64_tile_rows.  split_variant = 1 runs the split form as one launch per
 * system (each context's own split fields) instead of one for all.        */
int atrip_gpu_batch_set_tuning(atrip_gpu_batch *batch, const atrip_tuning *tuning);

/* ---------------------------------------------------------------------
 * No-allocation variant (no counterpart in the reference).
 *
 * For hosts that cannot call cudaMalloc: codes whose own pool allocator
 * owns all device memory, or frameworks that forbid device allocations on
 * their worker threads because cudaMalloc/cudaFree synchronise the device.
 * The caller passes device pointers to its column-major FP64 inputs (the
 * layout CTF's read_all returns) and to its outputs; the FP64 triples loop
 * runs without allocating anything.
 *
 * Scratch (work-queue cursor, per-CTA W buffers, reduction partials) lives
 * in one fixed 32 MiB __device__ array inside the library.  Every GPU that
 * loads the library holds that array until the process exits.  All calls
 * share it: each call clears what must start at zero, and calls whose
 * kernels overlap on the GPU (other streams, other host threads) race on it,
 * so serialise them.  Every call looks the array's device address up on
 * the current device (cudaGetSymbolAddress); the first call on a device
 * also loads the library's device code there, so make that first call
 * before any stream capture.  Limits: 1 <= No <= 64 (2 No^3 doubles of W
 * per CTA must fit in the array; at large No this also caps the number of
 * CTAs, e.g. 7 at No = 64), 1 <= Nv <= 1023.
 *
 * No checkpoint resume: unlike atrip_run_options there is no start_energy.
 * A caller resuming from a checkpoint passes first_iteration = the saved
 * Iteration and adds the saved energy to energies[0] itself.
 *
 * Tuples first_iteration .. max_iterations (inclusive; 0 = all) are run on
 * the current device, in `stream` (NULL = default stream); the call returns
 * after queueing the work.  Outputs (device memory, valid once the stream
 * has reached them):
 *   tuple_e[t - t0], tuple_ect[t - t0]  per-tuple energies, t0 = first tuple
 *                                       run (n = number of tuples in range)
 *   energies[0], energies[1]            energy and ct_energy of the range,
 *                                       final sign applied as in
 *                                       atrip_gpu_run (no checkpoint energy)
 * jijka/jabci may be NULL (then ct_energy == energy).                      */
typedef struct {
  const double *epsi, *epsa, *tai, *tabij, *vabij, *vijka, *vabci, *jijka, *jabci;
} atrip_device_inputs;

int atrip_gpu_run_fp64_noalloc(int32_t no, int32_t nv, const atrip_device_inputs *in,
                               int64_t first_iteration, int64_t max_iterations, int32_t ijkabc,
                               int32_t use_j, double *tuple_e, double *tuple_ect,
                               double *energies, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ATRIP_GB300_H */
