/*
 * gb300_ntt.h -- C ABI of the GB300 NTT library (libgb300ntt.so).
 *
 * The library re-implements, for one NVIDIA GB300 (sm_103a), the designs of
 * the AIE1 NTT artifact: radix-2 int16/int32 forward and inverse pipelines,
 * radix-4 and radix-8 int16 forward pipelines, and the stand-alone
 * bit-reversal and full-Barrett units.  Each design of the reference is an
 * ADF graph class whose constructor computes the twiddle/Barrett tables, whose
 * ports carry one polynomial per graph iteration, and whose lifecycle is
 * graph.init(); graph.run(N); graph.end() (src/project.cpp:161-164).  Here:
 *
 *   graph constructor + init()   ->  gbntt_plan_create()   (tables built once,
 *                                    kept resident in device memory)
 *   graph.run(N) over in_data /  ->  gbntt_execute()        (N polynomials per
 *   out_data ports                   call, one fused kernel launch)
 *   graph.end()                  ->  gbntt_plan_destroy()
 *
 * Conventions.  Polynomials are contiguous arrays of int16_t (int16 designs)
 * or int32_t (int32 designs); a batch is `batch` polynomials back to back.
 * Forward transforms take natural-order input and return bit-reversed output;
 * inverse transforms take bit-reversed input, return natural order, and omit
 * the factor n^-1 (reference README.md:157-160).  By default outputs are the
 * reference's partially reduced values, bit for bit; GBNTT_FLAG_CANONICAL
 * returns the same residues reduced to [0, q).  d_in is read-only; d_in ==
 * d_out (in place) is allowed.  Plans are immutable after creation and may be
 * used from several host threads and streams at once.  Every function returns
 * a gbntt_status; gbntt_last_error() gives a message for the calling thread.
 *
 * Launch ordering.  The per-plan launches (gbntt_execute's kernels) are
 * programmatic dependent launches: each kernel first signals that the next
 * grid on the stream may start, then waits for the previous grid's completion
 * and memory before it touches global memory, so calls that follow one another
 * on a stream start without a launch gap.  A caller's own kernel that follows
 * and is launched with cudaLaunchAttributeProgrammaticStreamSerialization must
 * call cudaGridDependencySynchronize() before it reads this library's outputs,
 * as the attribute requires; every other operation is ordered as usual.
 */
#ifndef GB300_NTT_H
#define GB300_NTT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBNTT_ABI_VERSION 1

/* Design kinds.  0..7 are the reference's NTT_CONFIG values
 * (src/project.cpp:35, :139-157; README.md:117-126). */
typedef enum gbntt_kind {
    GBNTT_R2_I16_FWD = 0,       /* NTT<n,q,w,...,TYPE_NTT_NO_to_BO>        src/ntt.h:43            */
    GBNTT_R2_I16_INV = 1,       /* NTT<n,q,w,...,TYPE_INTT_BO_to_NO>       src/ntt.h:43            */
    GBNTT_R4_I16_FWD = 2,       /* NTT_R4<n,q,w,...,FORWARD_CT_NO_TO_BO>   src/ntt_r4.h:30         */
    GBNTT_R8_I16_STAGE = 3,     /* NTT_R8<q,n,w>: one radix-8 stage        src/ntt_r8.h:22         */
    GBNTT_R2_I32_FWD = 4,       /* NTT_INT32<...,FORWARD_CT_NO_TO_BO>      src/ntt_int32.h:27      */
    GBNTT_R2_I32_INV = 5,       /* NTT_INT32<...,INVERSE_GS_BO_TO_NO>      src/ntt_int32.h:27      */
    GBNTT_BITREV_I16 = 6,       /* BITREVERSE<n>                           src/standalone_units.h:17 */
    GBNTT_FULL_BARRETT_I16 = 7, /* FULL_BARRETT_MULTIPLICATION<n,q,F>      src/standalone_units.h:40 */
    /* Designs the reference describes but does not ship as a graph: */
    GBNTT_R8_I16_FWD = 8,       /* all radix-8 stages chained, plus a radix-2/4 tail stage when
                                   log2 n is not a multiple of 3 (src/ntt_r8.h:15-19)           */
    GBNTT_R4_I16_INV = 9        /* bit-reversal + radix-4 forward with inverse twiddles, then
                                   bit-reversal to natural order (src/ntt_r4.h:18-20)           */
} gbntt_kind;

typedef enum gbntt_status {
    GBNTT_OK = 0,
    GBNTT_ERR_ARG = 1,        /* null pointer or argument out of range                         */
    GBNTT_ERR_LENGTH = 2,     /* n not a power of two or not supported by the design
                                 (src/auxiliary.h:11, src/kernels/bitreverse_kernels.cc:58)    */
    GBNTT_ERR_MODULUS = 3,    /* q not an odd prime candidate or above the lazy-reduction bound
                                 of the storage type (src/ntt.h:118, src/ntt_int32.h:16)       */
    GBNTT_ERR_ROOT = 4,       /* root is not of order exactly n ("ROOT is not correct",
                                 src/auxiliary.h:37,44)                                         */
    GBNTT_ERR_LAYERS = 5,     /* radix-4 needs an even number of radix-2 layers
                                 (src/ntt_r4.h:62-63)                                           */
    GBNTT_ERR_KIND = 6,       /* unknown design kind                                            */
    GBNTT_ERR_CUDA = 7,       /* CUDA runtime error (message in gbntt_last_error)               */
    GBNTT_ERR_NOMEM = 8,      /* device or host allocation failed                              */
    GBNTT_ERR_TIMEOUT = 9,    /* a bounded wait ran out                                         */
    GBNTT_ERR_ADMISSION = 10  /* a request could not be admitted (not enough free memory)       */
} gbntt_status;

/* Plan flags
 *
 * GBNTT_FLAG_CANONICAL: outputs are residues in [0, q) of the exact transform
 * of the inputs (each input coefficient taken modulo q as a signed integer):
 * the forward DFT in bit-reversed order, the inverse (BO in, NO out) without
 * n^-1.  Those are the reference's outputs reduced modulo q wherever its
 * int16/int32 lanes do not wrap; they run on a kernel family of their own
 * (Shoup multiplication by precomputed quotients, lazily reduced 32-bit lanes,
 * one reduction at the end; twiddle tables built on the device), for every
 * transform design except the radix-8 single stage and the radix-8 chain with
 * the reference's float multipliers, and int32 moduli below 2^30.
 * GBNTT_FLAG_CANONICAL | GBNTT_FLAG_LANE_EXACT: the reference's own lane
 * arithmetic (the default partial kernels, wraps included) reduced to [0, q),
 * i.e. exactly the reference's residues also where its lanes wrap (full-range
 * int16 input to the radix-2 inverse, the radix-4 designs at q > 16383, int32
 * inverses at q >= 2^30); the designs the canonical family does not cover take
 * this form whenever GBNTT_FLAG_CANONICAL is set. */
#define GBNTT_FLAG_CANONICAL   0x1u  /* reduce outputs to [0, q)                                   */
#define GBNTT_FLAG_R8_EXACT    0x2u  /* exact K=31 radix-8 multipliers (default for R8_I16_FWD)    */
#define GBNTT_FLAG_R8_FLOAT    0x4u  /* the reference's float K=31 multipliers (src/twiddle.h:372;
                                        default for R8_I16_STAGE)                                  */
#define GBNTT_FLAG_NATURAL_ORDER 0x8u /* bit-reversal unit fused into the transform: forward designs
                                        return natural order, inverse designs take natural order   */
#define GBNTT_FLAG_SCALE_NINV 0x10u  /* int16 inverse designs: the full Barrett unit multiplying by
                                        n^-1 (src/project.cpp:154) fused into the store (also the
                                        canonical int32 inverse)                                    */
#define GBNTT_FLAG_LANE_EXACT 0x20u  /* with GBNTT_FLAG_CANONICAL: the reference's lane arithmetic,
                                        reduced to [0, q) (no effect without it)                   */

typedef struct gbntt_plan gbntt_plan;

/* Builds a plan: validates (kind, n, q, root), computes the reference's
 * tables on the host, uploads them to the current device (they stay resident
 * until gbntt_plan_destroy).  `root` is a primitive n-th root of unity modulo
 * q (the inverse designs invert it themselves, like src/twiddle.h:80,112).
 * `factor` is the multiplier of GBNTT_FULL_BARRETT_I16 (e.g. n^-1 mod q,
 * src/project.cpp:154); ignored otherwise.  BITREV_I16 ignores q and root. */
int gbntt_plan_create(gbntt_plan** plan, int kind, uint32_t n, int64_t q, int64_t root,
                      int64_t factor, uint32_t flags);

/* Releases the plan's device tables.  NULL is accepted. */
int gbntt_plan_destroy(gbntt_plan* plan);

/* Transforms `batch` polynomials held in device memory, asynchronously on
 * `stream` (a cudaStream_t; NULL = legacy default stream).  One kernel launch
 * per call, except the int32 designs with n >= 2^16 (up to 2^22), which run
 * two passes (column and row sub-transforms) per chunk of polynomials (at most
 * 96 MiB, which stays in L2 between the passes; the canonical four-step's
 * column pass moves 2D tiles with the Tensor Memory Accelerator and its row
 * pass applies the four-step twist).  The environment variable GBNTT_FOURSTEP_MIN_L (14, 15 or 16, read
 * once per process) moves the canonical int32 plans of n >= 2^that length to
 * the four-step (default 16: n = 2^14 and 2^15 run one CTA per polynomial);
 * GBNTT_FOURSTEP_CHUNK_MB (8 .. 120, read once) sets the chunk size of both
 * two-pass schedules. */
int gbntt_execute(const gbntt_plan* plan, const void* d_in, void* d_out, uint64_t batch,
                  void* stream);

/* Synchronous: GBNTT_ERR_TIMEOUT if a bounded wait in an earlier launch of
 * this plan ran out (the TMA tile loads of the canonical int32 four-step,
 * n >= 2^16; the other designs have no waits); the call clears it. */
int gbntt_plan_status(const gbntt_plan* plan);

/* Same, on host buffers, and waits for the stream; serialised per plan.  When
 * both buffers are page-locked and mapped into the device's address space
 * (cudaHostAlloc / cudaHostRegister memory, 16-byte aligned) and the design
 * has a persistent-kernel form (all but the radix-4 inverse, the radix-8
 * stage, the bit-reversal and full Barrett units and int32 n >= 2^14), the
 * zero-copy persistent kernel reads and writes them directly over the
 * host-device link; its scratch (a descriptor and tile counters) is allocated
 * on the first such call, and a call on the same buffers and count as the
 * previous one reuses the descriptor already on the device.  Otherwise the
 * inputs are copied to device staging memory owned by the plan, transformed
 * and copied back. */
int gbntt_execute_host(gbntt_plan* plan, const void* h_in, void* h_out, uint64_t batch,
                       void* stream);

/* Plan properties. */
#define GBNTT_Q_N           0  /* n                                    */
#define GBNTT_Q_MODULUS     1  /* q                                    */
#define GBNTT_Q_ELEM_BYTES  2  /* 2 (int16 designs) or 4 (int32)       */
#define GBNTT_Q_STAGES      3  /* pipeline stages of the reference design (tiles) */
#define GBNTT_Q_KIND        4
#define GBNTT_Q_TABLE_BYTES 5  /* device bytes held by the plan's tables */
int gbntt_plan_query(const gbntt_plan* plan, int what, int64_t* value);

/* Host-side tables, without any CUDA call (for checking the table code on a
 * machine without a GPU).  which = 0: the device twiddle table as (tw, w')
 * pairs flattened; 1: the scalar constants.  Writes at most cap values and
 * stores the full length in *len. */
int gbntt_host_tables(int kind, uint32_t n, int64_t q, int64_t root, int64_t factor,
                      uint32_t flags, int which, int64_t* dst, int64_t cap, int64_t* len);

/* ---- batches: many polynomials of several designs in one persistent launch ----
 *
 * A batch is a fixed list of segments (plan, device input, device output,
 * number of polynomials).  gbntt_batch_execute transforms all of them with one
 * persistent kernel launch per storage type (int16 designs, int32 designs):
 * tiles of polynomials are handed out dynamically, largest n first, and move
 * between HBM and shared memory as bulk (TMA) copies, double-buffered.
 * Segments the persistent kernel does not cover (bit-reversal, full Barrett,
 * the radix-8 single stage, the radix-4 inverse, in-place segments, n outside
 * its range) run as their plans' own launches after it, on the same stream.
 * The batch owns a few words of device scratch (tile counter), so launches of
 * one batch must not overlap; different batches may run concurrently. */
typedef struct gbntt_segment {
    const gbntt_plan* plan;
    const void* d_in;
    void* d_out;
    uint64_t count;
} gbntt_segment;

typedef struct gbntt_batch gbntt_batch;

/* flags: GBNTT_BATCH_NO_TUNE skips the autotuner, which otherwise times every
 * persistent-kernel configuration (coefficients per thread, hence threads
 * and CTAs per transform and polynomials per tile, and resident CTAs per SM)
 * on the batch itself at creation and keeps the fastest.  A batch whose
 * inputs and outputs fit in L2 is timed from HBM: creation then briefly
 * allocates twice the L2 size of scratch to evict it between the timed
 * launches (without room for it, the launches are timed back to back).
 * Creation then writes the segments' outputs. */
#define GBNTT_BATCH_NO_TUNE 0x1u
int gbntt_batch_create(gbntt_batch** batch, const gbntt_segment* segs, uint32_t nsegs, uint32_t flags);
int gbntt_batch_execute(gbntt_batch* batch, void* stream);
/* The same launches captured once in a CUDA graph and replayed. */
int gbntt_batch_graph_launch(gbntt_batch* batch, void* stream);
/* Host buffers, waiting for the stream.  When the buffers of every segment the
 * persistent kernel covers are page-locked and mapped into the device's
 * address space (cudaHostAlloc / cudaHostRegister memory, 16-byte aligned),
 * the zero-copy form of the persistent kernel reads and writes them directly
 * over the host-device link, so inbound and outbound traffic overlap (one
 * launch per storage type; h_in[i] == h_out[i] allowed; a call on the same
 * buffers as the previous successful one reuses the descriptors already on
 * the device); the other segments are copied through their device buffers.
 * Otherwise copies h_in[i] into
 * segment i's device input, runs the batch (graph replay) and copies every
 * segment's device output to h_out[i].  Not concurrent with other launches of
 * the same batch. */
int gbntt_batch_execute_host(gbntt_batch* batch, const void* const* h_in, void* const* h_out, void* stream);
/* Rebinds a segment's buffers (no launch of the batch may be in flight). */
int gbntt_batch_set_io(gbntt_batch* batch, uint32_t seg, const void* d_in, void* d_out);
/* Synchronous: GBNTT_ERR_TIMEOUT if a tile load of an earlier launch ran out
 * of its bounded wait (the error is cleared by the call). */
int gbntt_batch_status(gbntt_batch* batch);
/* Poll limit of the bounded wait for each tile load of the persistent kernel
 * (batches, the no-alloc call, the serving loop), for launches enqueued after
 * the call (a batch's CUDA graph keeps the limit it was captured with).  The
 * default is GBNTT_WAIT_POLLS_DEFAULT; 0 makes every such wait give up at once.
 * A tile whose wait runs out makes its CTA record GBNTT_ERR_TIMEOUT (reported
 * by gbntt_batch_status, gbntt_noalloc_status and the server's waits), let its
 * copies in flight land (those waits keep the default limit) and stop.  Small
 * limits are for tests of that failure path.  No counterpart in the reference
 * (AIE graphs have no runtime error channel). */
#define GBNTT_WAIT_POLLS_DEFAULT 4194304u
int gbntt_set_wait_limit(uint32_t polls);
#define GBNTT_BQ_LAUNCHES 0   /* kernel launches per execute            */
#define GBNTT_BQ_TILES    1   /* tiles of the persistent launches        */
#define GBNTT_BQ_GRID     2   /* CTAs of the largest persistent launch   */
#define GBNTT_BQ_SMEM     3   /* dynamic shared memory per CTA (bytes)   */
#define GBNTT_BQ_EL16     4   /* log2 coefficients per thread chosen for the int16 launch */
#define GBNTT_BQ_FAMSET   5   /* design families compiled into the chosen int16 kernel (bit mask) */
#define GBNTT_BQ_CTA      6   /* threads per CTA of the chosen int16 kernel */
#define GBNTT_BQ_OCC      7   /* resident CTAs per SM the chosen int16 kernel's registers are budgeted
                                 for (0: the width's default) */
/* Setting the environment variable GBNTT_TUNE_LOG=1 prints the autotuner's
 * timing of every candidate configuration to stderr at batch creation;
 * GBNTT_TUNE_FORCE="<log2 coefficients per thread>,<CTAs per SM, 0 = default>"
 * pins the choice among the candidates (the timing launches still run). */
int gbntt_batch_query(const gbntt_batch* batch, int what, int64_t* value);
int gbntt_batch_destroy(gbntt_batch* batch);

/* ---- batch execution that allocates nothing ----
 * No counterpart in the reference (its graphs own all their memory at compile
 * time).  gbntt_batch_create allocates device memory for a batch's tile
 * descriptors and counters; callers that cannot allocate device memory when
 * they transform (an application that owns every device buffer through its own
 * allocator or arena, a serving loop that must not synchronise the device with
 * cudaMalloc/cudaFree in the middle of a request) use this call instead.  It
 * runs the same persistent kernel on up to GBNTT_NOALLOC_MAX_SEGMENTS segments
 * (plans created beforehand, caller-owned device buffers), keeping descriptors
 * and counters in one fixed static device array (about 8 KB, held on every
 * GPU that loads the library until the process exits).  More segments are
 * rejected with GBNTT_ERR_ARG; every segment's configuration is checked before
 * anything is enqueued.  The first call on a device looks the array up
 * (cudaGetSymbolAddress) with that device current; make that first call before
 * any stream capture.  The descriptors reach the array through a one-CTA kernel
 * whose launch parameters carry them (no copy from host memory).  Every call
 * reuses the array and resets its tile counters, so calls whose work overlaps
 * on the GPU (different streams, no ordering between them) race; serialise
 * them on one stream.  No autotuning: the narrowest compiled configuration
 * covering the segments' designs and lengths, with the most resident CTAs
 * among those, is used. */
#define GBNTT_NOALLOC_MAX_SEGMENTS 16
int gbntt_batch_execute_noalloc(const gbntt_segment* segs, uint32_t nsegs, void* stream);
/* Synchronous, on the current device: GBNTT_ERR_TIMEOUT if a tile load of an
 * earlier gbntt_batch_execute_noalloc launch ran out of its bounded wait (its
 * outputs are then incomplete); the call clears the error words it reports. */
int gbntt_noalloc_status(void);

/* ---- serving loop: continuous batching of transform requests ----
 * Requests (a plan of the server, host input, host output, polynomial count)
 * may be submitted from any host thread.  A worker thread admits them while
 * the server's device arena has room (its size is the configured budget,
 * capped at half of the HBM free at creation), groups the waiting ones by
 * plan into a micro-batch per free stream slot, and overlaps the copies and
 * kernels of up to `slots` micro-batches.  A micro-batch is one in-place
 * launch of the persistent kernel per storage type covering all its plan
 * groups (int32 n >= 2^16 and the radix-4 inverse, bit-reversal and full
 * Barrett designs: their plans' own launches).  Page-locked host buffers
 * mapped into the device's address space are read and written by a gather and
 * a scatter kernel (no per-request copy call); other host memory goes through
 * one cudaMemcpyAsync per direction.  Both buffers of a request must stay
 * valid and untouched until its wait returns.  Requests larger than the whole
 * arena are refused (their wait returns GBNTT_ERR_ADMISSION).  Latency =
 * submit to completion as seen by the worker.  Radix-8 stage plans (which
 * cannot run in place) are rejected at creation. */
typedef struct gbntt_server gbntt_server;
typedef struct gbntt_server_config {
    uint32_t slots;                   /* concurrent micro-batches (streams); 0 = 8 */
    uint32_t max_requests_per_batch;  /* 0 = 4096                                  */
    uint64_t device_bytes;            /* arena budget; 0 = 1 GiB                   */
} gbntt_server_config;
typedef struct gbntt_server_stats {
    uint64_t completed, refused, polynomials, microbatches, launches;
    double p50_us, p99_us, max_us;    /* request latency percentiles (nearest rank) */
    double polys_per_s;               /* polynomials completed per second           */
    uint64_t arena_bytes, peak_arena_bytes;
} gbntt_server_stats;
int gbntt_server_create(gbntt_server** server, const gbntt_plan* const* plans, uint32_t nplans,
                        const gbntt_server_config* cfg);
int gbntt_server_submit(gbntt_server* server, uint32_t plan, const void* h_in, void* h_out, uint64_t count,
                        uint64_t* ticket);
int gbntt_server_wait(gbntt_server* server, uint64_t ticket, uint32_t timeout_ms);
int gbntt_server_drain(gbntt_server* server, uint32_t timeout_ms);
int gbntt_server_get_stats(gbntt_server* server, gbntt_server_stats* stats, int reset);
int gbntt_server_destroy(gbntt_server* server);
/* Open-loop load generator: submits request i at arrival_us[i] microseconds
 * after the call (busy-waiting), writing its ticket to tickets[i]. */
int gbntt_server_submit_schedule(gbntt_server* server, uint64_t nreq, const uint32_t* plan,
                                 const void* const* h_in, void* const* h_out, const uint64_t* count,
                                 const double* arrival_us, uint64_t* tickets);
/* Checks the arena allocator and the percentile code on the host (no CUDA). */
int gbntt_server_selftest(void);

/* Total number of kernels this library has launched in this process. */
uint64_t gbntt_launch_count(void);

const char* gbntt_last_error(void);
const char* gbntt_status_string(int status);
int gbntt_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* GB300_NTT_H */
