/*
 * gpulucas.h -- C ABI of gpulucas_gb300, a GB300-native Lucas-Lehmer engine for
 * Mersenne numbers 2^p - 1 (irrational-base discrete weighted transform, FP64).
 *
 * The reference project (gpuLucas) is one executable whose routines are static
 * functions over file-scope globals (gpuLucas.cu:179-257).  Each entry point below
 * states which reference routine it replaces.  Conventions:
 *   - every function returns an int status: GL_OK (0) or a negative GL_ERR_* code;
 *     nothing here calls exit() (the reference exits on any CUDA error,
 *     cuda_safecalls.h:37-98, and on an out-of-range ratio, gpuLucas.cu:327-331);
 *   - a gl_plan owns all of its device memory and one CUDA stream; one host thread
 *     uses a plan at a time; there is no global state;
 *   - host buffers are owned by the caller.
 */
#ifndef GPULUCAS_H
#define GPULUCAS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GL_OK 0
#define GL_ERR_ARG -1        /* bad argument (p, N, pointer, option) */
#define GL_ERR_RATIO -2      /* p/N outside the carry-depth table (setSliceAndDice) */
#define GL_ERR_SIZE -3       /* N not even, not 2^a 3^b 5^c 7^d, or no FFT layout */
#define GL_ERR_CUDA -4       /* a CUDA runtime call failed */
#define GL_ERR_NOMEM -5      /* device or host allocation failed / over budget */
#define GL_ERR_ROUNDOFF -6   /* max round-off |x - rint(x)| reached the error limit */
#define GL_ERR_OVERFLOW -7   /* a product left the range the carry slices cover */
#define GL_ERR_NODEVICE -8   /* no CUDA device */
#define GL_ERR_IO -9         /* checkpoint file could not be read or written */
#define GL_ERR_CHECKPOINT -10 /* checkpoint does not match this test */
#define GL_ERR_STATE -11     /* call not valid in the plan's current state */
#define GL_ERR_TOO_LARGE -12 /* N above the limit of the no-allocation entry point */
#define GL_ERR_TIMEOUT -13   /* a bounded wait in a kernel ran out (an asynchronous copy never
                                completed); the kernel returned without computing */

/* execution forms */
#define GL_MODE_FUSED 0      /* 3 fused kernels per iteration (the product form) */
#define GL_MODE_PLAIN 1      /* one kernel per reference step (comparison form) */

typedef struct gl_plan gl_plan;

typedef struct {
    int mode;              /* GL_MODE_FUSED or GL_MODE_PLAIN */
    int device;            /* CUDA device ordinal */
    double error_limit;    /* abort when max round-off >= this (default 0.4) */
    int check_every;       /* read the round-off status every K iterations (default 1000) */
    int use_graphs;        /* capture iteration batches in CUDA graphs (default 1) */
    int fft_h;             /* 0 = automatic; else force the column length H of M = W*H */
    int cols_per_cta;      /* 0 or 1 (the column passes take one column per CTA) */
    int autotune;          /* 1 (default): time the best few layouts once per N per process */
    int batch_layout;      /* 1: layout for running inside a batch (total work, no timing) */
    int high_priority;     /* stream priority of the plan (or batch): 0 normal, 1 the device's
                              highest, 2 between the two; higher-priority blocks are
                              scheduled ahead of other work */
    int max_radix_col;     /* fused form: largest radix of the column / row line plans */
    int max_radix_row;     /* (8, 4 or 2; 0 = 8, or the autotuner's choice) */
    int resident;          /* fused form, short lengths: run whole check intervals in one
                              thread-block cluster holding the test in shared memory;
                              0 = by default up to N = 4096 (where it is faster),
                              1 = require (N <= 32768), -1 = never */
    int col_inplace;       /* fused form: column passes with in-place line DFTs (one buffer,
                              four CTAs per SM); 2: also bulk-copy the inverse pass's weights
                              into shared memory; 3: two columns per CTA, one per half of the
                              block, so that one half's dicing or rounding overlaps the other
                              half's DFT; 4: 3 for the forward pass, 2 for the inverse pass;
                              0 = the autotuner decides, -1 = never */
    int row_pass;          /* fused form: the row pass compiled for any radix (-1), or, for
                              row plans of radices 4, 3 and 2 only, compiled for those (1:
                              stage values in shared memory; 2: read through L1, so more
                              CTAs fit an SM); 0 = the autotuner decides */
} gl_plan_opts;

typedef struct {
    int p, N;
    int lo_bits, hi_bits;  /* floor(p/N), floor(p/N)+1 (initConstantSymbols, gpuLucas.cu:222-237) */
    int carry_depth;       /* n of llintToIrrBal<n> (setSliceAndDice, gpuLucas.cu:323-343) */
    int mode;
    int fft_w, fft_h;      /* N/2 = fft_w * fft_h complex points */
    int cols_per_cta;      /* columns per CTA of the forward column pass (1, or 2 with
                              col_inplace 3 or 4) */
    int radix_w[8], radix_h[8];
    int threads_col, threads_row;  /* CTA sizes of the column and row passes */
    int smem_col, smem_row;        /* dynamic shared memory bytes of those passes */
    size_t device_bytes;   /* device memory held by the plan */
    int resident_ctas;     /* CTAs of the resident form's cluster, 0 if not used */
    int resident_smem;     /* its shared memory per CTA */
    int col_variant;       /* fused form: the column passes as a col_inplace value (-1 two
                              buffers, 1 in place, 2 + prefetched weights, 3 two columns per
                              CTA, 4 two columns forward + prefetched weights inverse) */
    int row_variant;       /* fused form: the row pass as a row_pass value (-1, 1, 2) */
} gl_plan_info;

typedef struct {
    int64_t iterations;    /* iterations done by this call */
    int64_t total_iterations; /* iterations since S0 = 4 */
    double max_roundoff;   /* max |x - rint(x)| seen by this call (checked iterations) */
    double ms;             /* device time of the call, CUDA events */
    int status;            /* GL_OK, GL_ERR_ROUNDOFF or GL_ERR_OVERFLOW */
} gl_iter_report;

typedef struct {
    int p, N;
    int64_t iterations;    /* LL iterations done (p - 2 for a full test) */
    int is_prime;          /* residue == 0 mod 2^p - 1 after p - 2 iterations */
    int is_zero;           /* exact zero test of the current residue */
    uint64_t res64;        /* low 64 bits of S_k mod 2^p - 1 */
    double max_roundoff;   /* over the run */
    double ms;             /* device time */
} gl_result;

/* --- options and plans ------------------------------------------------ */
int gl_default_opts(gl_plan_opts* opts);

/* Replaces initConstantSymbols + setSliceAndDice + mallocArrays + computeBitsPerWord(Vectors)
 * + computeWeightVectors + cufftPlan1d (gpuLucas.cu:222-237, 323-343, 948-1029, 673-714).
 * N == 0 picks N with gl_find_signal_size. */
int gl_plan_create(int p, int N, const gl_plan_opts* opts, gl_plan** plan);
/* findSignalSize (gpuLucas.cu:1064-1187): FFT length for exponent p.  Candidates are the
 * even N with N/2 = 2^a 3^b 5^c 7^d (b <= 5, c <= 3, d <= 2) from the smallest the carry
 * table accepts (p/N < 22) upward; each gets a 100-iteration round-off trial of the real
 * test and is accepted below 0.30 (ERROR_LIMIT, gpuLucas.cu:176); among the accepted ones
 * within 15 % of the smallest, the fastest autotuned iteration wins.  *ms_per_iter and
 * *max_roundoff (either may be NULL) describe the choice. */
int gl_find_signal_size(int p, const gl_plan_opts* opts, int* N_out, double* ms_per_iter, double* max_roundoff);
/* Replaces freeArrays (gpuLucas.cu:1031-1057). */
int gl_plan_destroy(gl_plan* plan);
int gl_plan_get_info(const gl_plan* plan, gl_plan_info* info);
/* The layout gl_plan_create would choose for (p, N, opts), without touching a GPU. */
int gl_plan_describe(int p, int N, const gl_plan_opts* opts, gl_plan_info* info);

/* Replaces loadValue4ToFFTarray (gpuLucas.cu:718-726): state := S0 = 4. */
int gl_reset(gl_plan* plan);

/* Runs `iters` LL iterations: the loop body mersenneIter<check,0> (gpuLucas.cu:845-942)
 * with the round-off check of mersenneTest (gpuLucas.cu:1399-1410), aborting with
 * GL_ERR_ROUNDOFF at the plan's error limit. */
int gl_iterate(gl_plan* plan, int64_t iters, gl_iter_report* report);

/* Asynchronous forms for callers that time or overlap work themselves: enqueue
 * iterations on the plan's stream without waiting; read (and wait for) the status. */
int gl_plan_stream(gl_plan* plan, void** cuda_stream);
int gl_enqueue(gl_plan* plan, int64_t iters);
int gl_sync_status(gl_plan* plan, gl_iter_report* report);
/* kernel launches one iteration issues (3 for the fused form) */
int gl_launches_per_iteration(const gl_plan* plan);
/* Fused form only: run `iters` iterations launching each kernel between CUDA events
 * on the plan's stream; ms_out[i] = average ms of kernel i (k_col_fwd, k_row_sq,
 * k_col_inv); names (may be NULL) receives their names, *nk the count. */
int gl_profile_kernels(gl_plan* plan, int iters, double* ms_out, const char** names, int* nk);

/* The state after the last iteration. */
int gl_get_products(gl_plan* plan, int64_t* ll_out);                     /* llint_signal, N int64 */
int gl_get_carry_state(gl_plan* plan, int32_t* digit_out, int8_t* hi_out); /* i_signal, i_hiBitArr */
/* Set the loop-carried products (llint_signal) and the iteration count; the next
 * iteration, or gl_get_carry_state, dices them with llintToIrrBal<n>
 * (IrrBaseBalanced.cu:52-110). */
int gl_set_products(gl_plan* plan, const int64_t* ll, int64_t iterations);
/* For callers that keep the state in host memory: loads the carry-save state (digit,
 * hi; N each, host buffers), runs `iters` iterations, and writes the resulting state
 * back, with one synchronisation for the whole call (the round-off of these iterations
 * is checked once, at the end).  digit_in/hi_in may alias digit_out/hi_out; pinned
 * buffers copy at the CPU link's full rate.  With pinned buffers and iters == 1 the step
 * runs as one CUDA graph kept by the plan, whose last kernel stores the state and the
 * status straight into the mapped output buffers (as gl_iterate_host_words below). */
int gl_iterate_host(gl_plan* plan, const int32_t* digit_in, const int8_t* hi_in, int64_t iters,
                    int32_t* digit_out, int8_t* hi_out, gl_iter_report* report);
/* The same with the state as carry-added words, 4 bytes per word instead of 5: word j is
 * digit[j] + hi[j-1] (mod N), the integer that loadIntToDoubleIBDWT weights into the
 * next FFT input (gpuLucas.cu:730-766) and that addPseudoBalanced forms
 * (IrrBaseBalanced.cu:117-125).  Loading words w continues exactly as the carry-save
 * state it came from (the next FFT input is the same), and the words returned are the
 * carry-save state after the iterations with its carries added.  words_in may alias
 * words_out.  With pinned buffers and iters == 1 (a caller stepping one iteration at a
 * time) the whole step runs as one CUDA graph, built on the first call for these buffers
 * and kept by the plan; in it the kernel that forms the words stores them (and the
 * round-off status) straight into the mapped output buffer, so that transfer runs under
 * the kernel instead of as a copy after it.  Both buffers must hold N words until the
 * call returns. */
int gl_iterate_host_words(gl_plan* plan, const int32_t* words_in, int64_t iters, int32_t* words_out,
                          gl_iter_report* report);
/* Set a carry-save state (balanced digits + int8 carries) and its iteration count. */
int gl_set_carry_state(gl_plan* plan, const int32_t* digit, const int8_t* hi, int64_t iterations);

/* addPseudoBalanced + rebalanceIrrIntSEQGPU + print_residue + zero test
 * (IrrBaseBalanced.cu:117-169, gpuLucas.cu:1288-1352, 1496-1512): rebalanced digits
 * (may be NULL), Res64 and the exact zero test of the current state. */
int gl_get_residue(gl_plan* plan, int32_t* digits_out, uint64_t* res64, int* is_zero);

/* --- checkpoints in the reference's file format --------------------------- */

/* writeCheckpoint (gpuLucas.cu:1641-1665): char[16] "gpuLucas", char[16] "0.9.4", int p,
 * int N, int iter, then N doubles of the weighted FFT input A[j](digit[j] + hi[j-1])
 * (d_signal).  iter follows the reference's loop count: a state after k squarings is
 * written with iter = k + 1.  The old file is kept as path.bak; the new one is written
 * to a temporary name and renamed, so a crash never leaves a torn checkpoint. */
int gl_checkpoint_write(gl_plan* plan, const char* path);
/* readCheckpoint (gpuLucas.cu:1569-1639): header checks (name "gpuLucas", p), N, the
 * squarings done (iter - 1) and, if digits_out is not NULL (N int32), the digit vector
 * round(d[j] / A[j]).  Falls back to path.bak when path is missing or unreadable.
 * GL_ERR_IO / GL_ERR_CHECKPOINT on failure; needs no GPU. */
int gl_checkpoint_read(const char* path, int p, int* N_out, int64_t* iterations_out, int32_t* digits_out);
/* Resume a plan (same p and N) from a checkpoint: the next iteration's FFT input equals
 * the saved d_signal bit for bit, as the reference's resume (gpuLucas.cu:1361-1363). */
int gl_plan_resume(gl_plan* plan, const char* path);

/* --- reference entry points (README: errorTest / mersenneTest) ---------- */

/* errorTrial (gpuLucas.cu:1192-1282) as README's errorTest(p, N): runs
 * clamp(p/10000, 100, 2500) iterations (gpuLucas.cu:529-541) and returns the average
 * ms per iteration, or -1 when the round-off reached the limit (gpuLucas.cu:903-907). */
float errorTest(int testPrime, int signalSize);
/* mersenneTest (gpuLucas.cu:1358-1551) as README's mersenneTest(p, N): full p-2 iteration
 * test.  Returns 1 if 2^p - 1 is prime, 0 if composite, a negative GL_ERR_* on error. */
int mersenneTest(int testPrime, int signalSize);
/* setSliceAndDice (gpuLucas.cu:323-343): carry depth n for p/N, extended to ratio 21;
 * GL_ERR_RATIO for ratio >= 22. */
int setSliceAndDice(int testPrime, int signalSize);

/* Plan-based forms with full results. */
int gl_error_test(int p, int N, const gl_plan_opts* opts, int iters, gl_iter_report* report);
int gl_mersenne_test(gl_plan* plan, int64_t iters, gl_result* result);

/* --- batches: many tests advanced together ------------------------------- */

/* No counterpart in the reference (it runs one test per process).  Smallest even N with
 * N/2 = 2^a 3^b 5^c 7^d (any exponents) and p/N <= max_bits_per_word (the batch
 * configuration uses 19.5). */
int gl_smallest_signal_size(int p, double max_bits_per_word, int* N_out);
/* Smallest such N with p/N <= 19.2 - 0.26 log2(N / 163840): the word size at which the
 * fused kernels' measured max round-off over 300 iterations from S0 = 4 stays at or
 * below 0.125 on GB300 (5760 <= N <= 2621440), leaving the 0.4 limit a factor three for
 * the tail of long runs.  A host-only length rule for servers that cannot afford
 * gl_find_signal_size's trial runs. */
int gl_safe_signal_size(int p, int* N_out);
/* A fast length in [gl_safe_signal_size, (1 + slack) x that]: the smallest whose odd
 * part is 1 or 3 (measured fastest: 98304 = 2^15 3 takes 33 us per iteration where
 * 84672 = 2^6 3^3 7^2 takes 41 us), else the cheapest under the layout cost model.
 * Host only. */
int gl_fast_signal_size(int p, double slack, int* N_out);

typedef struct gl_batch gl_batch;
typedef struct {
    int ntests;
    int col_units, row_units;      /* CTAs per column-pass / row-pass launch */
    int threads_col, threads_row;
    int smem_col, smem_row;
    size_t device_bytes;
    int64_t iterations;            /* iterations every test has done */
} gl_batch_info;

/* One fused-form plan per test (N[i] == 0: gl_smallest_signal_size(p[i], 19.5)), a
 * device descriptor table of their arguments, and unit maps so that three launches
 * advance every test by one iteration (64-iteration CUDA graphs).  opts: device,
 * error_limit, check_every. */
int gl_batch_create(const int* p, const int* N, int ntests, const gl_plan_opts* opts, gl_batch** batch);
/* A batch over existing fused-form plans of the same device, which it does not own: a
 * server rebuilds the batch when its set of live tests changes without rebuilding any
 * test's tables.  The plans must outlive the batch and are advanced only through it
 * while it exists. */
int gl_batch_create_from_plans(gl_plan* const* plans, int nplans, const gl_plan_opts* opts, gl_batch** batch);
int gl_batch_destroy(gl_batch* batch);
/* All tests advance `iters` iterations; per-test round-off is checked every check_every.
 * Returns the worst status (GL_ERR_ROUNDOFF / GL_ERR_OVERFLOW name some test). */
int gl_batch_iterate(gl_batch* batch, int64_t iters, gl_iter_report* report);
int gl_batch_stream(gl_batch* batch, void** cuda_stream);
int gl_batch_enqueue(gl_batch* batch, int64_t iters);
int gl_batch_sync_status(gl_batch* batch, gl_iter_report* report);
/* 1 if everything enqueued on the batch has finished, 0 if not, < 0 on error (no wait). */
int gl_batch_query(gl_batch* batch);
/* Test `index`: Res64 / zero test of its current state, its max round-off and status. */
int gl_batch_result(gl_batch* batch, int index, gl_result* result, int* status);
/* Round-off and status of one test as of the last status read (gl_batch_iterate or
 * gl_batch_sync_status); no device work. */
int gl_batch_test_status(const gl_batch* batch, int index, double* max_roundoff, int* status);
int gl_batch_get_info(const gl_batch* batch, gl_batch_info* info);
int gl_batch_test_info(const gl_batch* batch, int index, gl_plan_info* info);

/* --- serving: a request loop with continuous batching -------------------- */

/* No counterpart in the reference (one test per process, gpuLucas.cu:374-639).  A
 * server owns a background thread that admits submitted requests against an HBM budget
 * and a slot limit (arrival order), builds each test's plan on worker threads, and
 * advances the live tests in batches on separate streams: the lead lane (the device's
 * highest stream priority) runs alone the long test with the most iterations left, the
 * chain lane (next priority) the other full tests and requests of more than
 * chain_iterations, the bulk lane (normal priority) the rest.  A lane's batch is rebuilt from the live plans when its
 * membership changes; each step is bounded by step_ms of GPU time and by the next
 * completion or Res64 checkpoint.  A test whose round-off reaches error_limit restarts
 * from S0 = 4 at the next larger length (at most `retries` times), as the reference
 * aborts such a run (gpuLucas.cu:1470-1479).  Residues stay on the device; finished
 * tests report Res64 / zero test and free their memory. */
typedef struct gl_server gl_server;

typedef struct gl_server_opts {
    int device;
    double hbm_budget_bytes;     /* device bytes the live tests may hold */
    int max_active;              /* live tests at most */
    double step_ms;              /* GPU time per lane step at most */
    int64_t checkpoint_every;    /* Res64 of full tests every this many iterations (0: never) */
    double max_bits_per_word;    /* > 0: smallest length with p/N <= this; else gl_fast_signal_size(p, 0.2) */
    int retries;                 /* restarts at a larger length after a round-off abort */
    int64_t chain_iterations;    /* requests longer than this go to the chain lane */
    int lanes;                   /* 3: lead + chain + bulk; 2: chain + bulk; 1: one batch */
    int build_threads;           /* host threads building plans */
    double error_limit;          /* round-off limit (0, 0.5] */
    int check_every;             /* round-off read-back interval inside a step */
    int reserved[8];
} gl_server_opts;

typedef struct gl_completion {
    int64_t id;
    int p, N;
    int64_t iterations;          /* iterations done (p - 2 for a full test) */
    int full;
    int status;                  /* GL_OK, GL_ERR_ROUNDOFF, GL_ERR_NOMEM (never fits), ... */
    int is_zero, is_prime;
    uint64_t res64;
    double max_roundoff;
    double arrival_s, admit_s, done_s;   /* seconds since gl_server_create */
    int attempts;                /* 1 + restarts at a larger length */
    int lane;                    /* 3 lanes: 0 lead, 1 chain, 2 bulk; 2: 0 chain, 1 bulk */
    int n_checkpoints;           /* Res64 checkpoints recorded (gl_server_checkpoints) */
    int reserved;
} gl_completion;

typedef struct gl_server_stats {
    double wall_s, lane_busy_s[3];
    int64_t steps[3], rebuilds[3];
    int peak_live[3];
    int live, queued, building;
    size_t bytes_in_use, peak_bytes;
    double flop_alg;             /* sum over steps of (5 N log2 N + 4 N) x iterations */
    int64_t submitted, completed;
} gl_server_stats;

/* The engine a server drives.  The default is the library's own plans and batches on
 * opts->device; an explicit engine lets the scheduling be exercised without a GPU.
 * Handles are opaque to the server.  finish() writes, per test of the batch in the
 * order given to batch(), the max round-off of that batch so far and a status;
 * batch()'s priority is a gl_plan_opts.high_priority level. */
typedef struct gl_server_engine {
    void* ctx;
    int (*signal_size)(void* ctx, int p, double max_bits_per_word, int above, int* N);
    int (*footprint)(void* ctx, int p, int N, size_t* bytes);
    int (*create)(void* ctx, int p, int N, void** test);
    void (*destroy)(void* ctx, void* test);
    int (*batch)(void* ctx, void* const* tests, int n, int high_priority, void** batch);
    void (*close_batch)(void* ctx, void* batch);
    int (*start)(void* ctx, void* batch, int64_t iters);
    int (*ready)(void* ctx, void* batch);          /* 1 done, 0 running, < 0 error */
    int (*finish)(void* ctx, void* batch, int n, double* max_roundoff, int* status);
    int (*res64)(void* ctx, void* test, uint64_t* res64, int* is_zero);
} gl_server_engine;

int gl_server_default_opts(gl_server_opts* opts);
int gl_server_create(const gl_server_opts* opts, const gl_server_engine* engine /* NULL: GPU */,
                     gl_server** server);
/* Queue a request; iterations 0 asks for the full p - 2 test.  Thread-safe. */
int gl_server_submit(gl_server* server, int64_t id, int p, int64_t iterations);
/* Move up to `max` completions (oldest first) into `out`; *n receives how many.  Waits
 * up to timeout_ms for the first one (0: no wait).  Thread-safe. */
int gl_server_poll(gl_server* server, gl_completion* out, int max, int* n, double timeout_ms);
/* Block until every submitted request has completed. */
int gl_server_drain(gl_server* server);
/* Res64 checkpoints (iteration, res64) of a completed request, up to `max`. */
int gl_server_checkpoints(gl_server* server, int64_t id, int64_t* iterations, uint64_t* res64, int max,
                          int* n);
int gl_server_get_stats(gl_server* server, gl_server_stats* stats);
/* Stops the loop (live tests are dropped) and frees everything.  Returns the loop's
 * first error, if any. */
int gl_server_destroy(gl_server* server);

/* --- no device allocation ------------------------------------------------ */

/* No counterpart in the reference.  For callers that may not call cudaMalloc (a
 * framework memory pool owns the device, or allocation would stall shared work):
 * runs `iters` LL iterations (the plain form, bit-identical products to a
 * GL_MODE_PLAIN plan) on the current device and `stream` (NULL = default stream),
 * from the products ll_in to the products ll_out (N int64 each, device memory owned
 * by the caller, natural word order; they may be the same buffer, but buffers that
 * overlap only in part return GL_ERR_ARG), and stores the maximum round-off in
 * *max_roundoff.  It allocates nothing: its work arrays, tables and status word live in
 * a static device array sized for N <= 65536 (about 3.3 MiB, held on every GPU that
 * loads the library until exit); larger N returns GL_ERR_TOO_LARGE.  A call with new
 * (p, N) uploads that test's tables into the array first.  The call is synchronous: it
 * returns after `stream` has finished the iterations, so it cannot be captured into a
 * CUDA graph (on a stream that is capturing it returns GL_ERR_ARG and enqueues
 * nothing).  All calls share the array; a lock held until the stream has finished keeps
 * the calls of one process from overlapping on the GPU.
 * Returns GL_ERR_ROUNDOFF at round-off >= 0.4 and GL_ERR_OVERFLOW as gl_iterate. */
int gl_iterate_noalloc(int p, int N, const int64_t* ll_in, int64_t* ll_out, int64_t iters,
                       double* max_roundoff, void* stream);

/* --- utilities ----------------------------------------------------------- */
const char* gl_error_string(int status);
int gl_version(void);        /* major*10000 + minor*100 + patch */
/* Self-test of the kernels' bounded waits: a kernel waits on a barrier nothing completes,
 * gives up after `tries` polls and reports it; returns GL_ERR_TIMEOUT when the timeout
 * path works (the device stays usable), GL_OK if the wait unexpectedly completed. */
int gl_selftest_bounded_wait(int device, int tries);
/* FP64 throughput probe (DFMA), for the roofline denominator: TFLOP/s counting an FMA
 * as 2 flops, measured on `device` for about `ms` milliseconds. */
int gl_probe_fp64_peak(int device, double ms, double* tflops);
/* FP64 issue rate of butterfly code: the twiddled radix-8 butterfly of the line DFTs
 * applied to register-resident points on all SMs for about `ms` milliseconds; FP64
 * instructions per second (one per DFMA, DADD or DMUL).  Compiled FP64 code with data
 * dependences issues below the DFMA probe's rate; this is the rate the FFT's own
 * instruction mix reaches when nothing else (shared memory, barriers) intervenes. */
int gl_probe_fp64_butterfly(int device, double ms, double* instr_per_s);

#ifdef __cplusplus
}
#endif
#endif /* GPULUCAS_H */
