/*
 * cumf_sgd.h - C ABI of the GB300-native batch-Hogwild SGD matrix-factorization path.
 *
 * Drop-in boundary for cuMF_SGD's single-GPU trainer.  Every entry point replaces one
 * reference interface (cited per declaration as file:line inside the cuMF_SGD project):
 *
 *   singleGPU/sgd.h:140        mf_problem read_problem(string)           -> cumf_read_problem
 *   singleGPU/sgd.h:141        mf_model* sgd_train(mf_problem*, ...)      -> cumf_train
 *   singleGPU/sgd_kernel.h:17  sgd_update_k128(Parameter, ...)            -> cumf_sgd_update
 *   singleGPU/main.cpp:231     save_model(mf_model const*, char const*)   -> cumf_save_model
 *   singleGPU/main.cpp:33      parse_argument(int, char**)                -> cumf_parse_args
 *   test/mf.cpp:3706           mf_load_model(char const*)                 -> cumf_load_model
 *   test/mf.cpp:3815           calc_rmse(mf_problem*, mf_model*)          -> cumf_rmse
 *   test/mf.cpp:3841-4044      calc_mae/gkl/logloss/accuracy/mpr/auc      -> cumf_evaluate
 *   data/netflix/transform.cpp ./transform file_name                      -> cumf_convert_text
 *
 * Conventions (differences from the reference are deliberate and listed here):
 *   - every call returns an int status (CUMF_OK == 0); nothing calls exit().  The message of
 *     the last failure on the calling thread is returned by cumf_last_error().
 *   - inputs are const: cumf_train copies the ratings and permutes/scales the copy (the
 *     reference mutates the caller's problem in place, sgd.cu:661,672).
 *   - no global RNG state: every random choice is a pure function of params.seed
 *     (the reference seeds from time(NULL) and clock(), sgd.cu:42,494).
 *   - device pointers in the cumf_dev_* / cumf_sgd_update family are plain addresses of
 *     device memory owned by the caller; `stream` is a cudaStream_t passed as void*.
 * Plain C types only; no C++ or torch types cross this boundary.
 */
#ifndef CUMF_SGD_H_
#define CUMF_SGD_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CUMF_ABI_VERSION 2

/* ---- status codes ---------------------------------------------------------------- */
enum {
    CUMF_OK = 0,
    CUMF_ERR_ARG = 1,      /* invalid argument / unsupported parameter                  */
    CUMF_ERR_IO = 2,       /* file missing, unreadable, short, or unwritable            */
    CUMF_ERR_FORMAT = 3,   /* malformed rating or model file (negative id, bad header)  */
    CUMF_ERR_CUDA = 4,     /* a CUDA runtime call failed                                */
    CUMF_ERR_NOMEM = 5,    /* host or device allocation failed                          */
    CUMF_ERR_RANGE = 6,    /* a rating index lies outside [0,m) x [0,n)                 */
    CUMF_ERR_TIMEOUT = 7,  /* a bounded device-side wait gave up                        */
    CUMF_ERR_NODEVICE = 8  /* no CUDA device visible                                    */
};

/* ---- factor storage precision (update arithmetic is always fp32) ------------------ */
enum {
    CUMF_FP16 = 0,     /* reference: half storage, round-to-nearest (warp32.h:89-99)    */
    CUMF_BF16 = 1,     /* bf16 storage, round-to-nearest                                 */
    CUMF_FP32 = 2,     /* fp32 storage                                                   */
    CUMF_BF16_SR = 3,  /* bf16 storage, stochastic rounding on every factor write        */
    CUMF_FP16_SR = 4   /* fp16 storage, stochastic rounding on every factor write        */
};

/* ---- records ---------------------------------------------------------------------- */
/* One rating: the 12-byte on-disk record {int32 u, int32 v, float32 r}.
 * Same layout as mf_node (singleGPU/sgd.h:79-83) and the file format (sgd.cu:251-253). */
typedef struct cumf_node {
    int32_t u;
    int32_t v;
    float r;
} cumf_node;

/* mf_problem (singleGPU/sgd.h:85-108), host side.  m = max u + 1, n = max v + 1, each at
 * least 1 (sgd.cu:202-203,256-257).  R is page-locked when `pinned` is 1. */
typedef struct cumf_problem {
    int32_t m;
    int32_t n;
    int64_t nnz;
    cumf_node *R;
    int32_t pinned;
    int32_t reserved_;
} cumf_problem;

/* Parameter (singleGPU/sgd.h:26-46) plus the build's additions.  cumf_default_params
 * fills the reference defaults (sgd.h:45). */
typedef struct cumf_params {
    int32_t k;             /* factor length; 32, 64, 128 or 256 (reference: 128 only)  */
    int32_t num_workers;   /* -s: Hogwild workers; rounded up to a multiple of 4; 0 = automatic
                              (cumf_auto_workers for the ratings of one grid block)         */
    int32_t u_grid, v_grid, x_grid, y_grid;   /* -u -v -x -y                            */
    int32_t ux, vy;        /* u_grid*x_grid, v_grid*y_grid (main.cpp:224-225)           */
    int32_t num_iters;     /* -t                                                        */
    int32_t gpu;           /* -g: device id, taken modulo the device count              */
    float lambda_p, lambda_q;  /* -l p[,q]                                              */
    float lrate;           /* -r: additive learning-rate floor (sgd_kernel.cu:146)      */
    float alpha, beta;     /* -a -b: lr(t) = alpha/(1+beta*t^1.5) + lrate               */
    /* additions ---------------------------------------------------------------------- */
    uint64_t seed;         /* seeds the id shuffle, factor init and sample draws        */
    int32_t precision;     /* CUMF_FP16 ...                                              */
    int32_t lanes;         /* lanes cooperating on one rating: 0 = auto, else 4..32     */
    int32_t quiet;         /* 1 = no informational stdout                               */
    int32_t epochs_per_launch; /* mode A: 0 = one launch per epoch (default); N > 0 = N
                                * epochs per launch while every worker is resident (N >=
                                * num_iters: one persistent launch, as sgd_kernel.cu:212-244) */
    int32_t verbose_epochs;    /* 1 = print one JSON line per epoch (needs a test set)  */
    int32_t prefetch;      /* L2 prefetch distance in records: -1 = tuned default, 0 = off */
    int32_t l2_hints;      /* L2 eviction hints: -1 = tuned default, 0 = off, 1 = on      */
    int32_t ring;          /* update kernel pipeline (see cumf_tuning.ring)               */
    int32_t tail_epochs;   /* the first tail_epochs epochs sample only records            */
    int32_t deterministic; /* 0 = batch-Hogwild (the reference); 1 = the stratified schedule
                              of cumf_dev_strata_epochs, bit-reproducible (mode A), with an
                              automatic grid; > 1 = that many user / item groups            */
    int64_t tail_start;    /* (tail_epochs) [tail_start, nnz) (e.g. newly added users'
                              ratings): those epochs update user rows only (item rows frozen) */
    float hot_rows;        /* batch-Hogwild, mode A: copies of the most-rated rows
                              (cumf_hot_rows_*) for this many expected workers per copy
                              (0.5 suits skewed item popularity); 0 = none, the default
                              (every rating updates its own row, as the reference)        */
    int32_t reserved_[3];
} cumf_params;

/* Launch tuning of the update kernel (the knobs the autotuner searches). */
typedef struct cumf_tuning {
    int32_t lanes;         /* lanes per rating: 0 = default for (k, precision)           */
    int32_t prefetch;      /* rows of record j+prefetch are pulled into L2 during record j;
                              -1 = default (2; see rows_copied), 0 = off, at most 15      */
    int32_t l2_hints;      /* -1 = default, 0 = none, 1 = ratings evict_first and factor
                              rows evict_last                                            */
    int32_t ring;          /* -1 = default, 0 = one record's rows in flight per worker (held
                              in registers), 1 = four records' rows in flight, staged by
                              cp.async in a shared-memory ring                            */
    int32_t freeze_q;      /* 1 = update user rows only; item rows are read, never written  */
    int32_t rows_copied;   /* 1 = the ratings name copies of the most-rated rows
                              (cumf_hot_rows_assign).  With rows_copied or freeze_q the
                              default prefetch is 0 unless P and Q together exceed twice the
                              L2 size                                                      */
    int32_t reserved_[2];
} cumf_tuning;

/* mf_model (singleGPU/sgd.h:110-138) as the model file holds it (main.cpp:247-266):
 * P is m x k and Q is n x k, row-major fp32, already unscaled and un-permuted. */
typedef struct cumf_model {
    int32_t fun;
    int32_t m;
    int32_t n;
    int32_t k;
    float b;
    int32_t pinned;        /* 1 if P and Q are page-locked (set by the allocator)       */
    float *P;
    float *Q;
} cumf_model;

/* Timings and counters of one cumf_train call (the reference prints update_per_sec from
 * clock(), sgd_kernel.cu:243-244; these are wall/CUDA-event times). */
typedef struct cumf_train_stats {
    double prep_ms;        /* H2D + stats + shuffle + scale + init                      */
    double train_ms;       /* SGD epochs only (CUDA events)                             */
    double export_ms;      /* fp16->fp32, unscale, un-permute, D2H                      */
    double total_ms;
    double updates_per_sec;/* nnz * num_iters / train time (reference convention)       */
    int64_t samples_per_epoch; /* workers * batches * 128                               */
    float mean, std_dev;   /* rating statistics (sgd.cu:78-96)                         */
    int32_t mode;          /* 0 = A (in HBM), 1 = B (u x v), 2 = C (x x y streaming)    */
    int32_t num_workers;
    int32_t lanes;
    int32_t hot_users, hot_items;  /* rows given copies (cumf_params.hot_rows)           */
    int32_t extra_rows;            /* rows added to P and Q for those copies               */
    int32_t reserved_[2];
} cumf_train_stats;

/* CLI arguments: Argument (singleGPU/sgd.h:48-77). */
typedef struct cumf_args {
    cumf_params param;
    char tr_path[1024];
    char va_path[1024];
    char model_path[1024];
} cumf_args;

/* ---- library ---------------------------------------------------------------------- */
int cumf_abi_version(void);
/* Message of the last failed call on this thread ("" if none). */
const char *cumf_last_error(void);
/* Reference defaults (singleGPU/sgd.h:45) plus seed 0, FP16, auto lanes, hot_rows 0 (no copies). */
int cumf_default_params(cumf_params *p);
/* parse_argument (singleGPU/main.cpp:33-227): same flags, same -s rounding, the same
 * default model path (<basename of train file>.model), u*v==1 forces x=y=1.  Long flags
 * added: --seed N, --precision fp16|bf16|fp32|bf16sr|fp16sr, --lanes N, --quiet,
 * --deterministic G, --hot-rows X (cumf_params.hot_rows; 0 = off).
 * Returns CUMF_ERR_ARG with the reference's message on bad input. */
int cumf_parse_args(int argc, char **argv, cumf_args *out);

/* ---- host I/O --------------------------------------------------------------------- */
/* read_problem (singleGPU/sgd.cu:190-335): single file, or shards path0..path79 read in
 * parallel when path0 exists.  nnz = size/12 (a trailing partial record is ignored, as in
 * the reference).  Negative ids are rejected (CUMF_ERR_FORMAT).  pinned=1 allocates R
 * page-locked (the reference always does, sgd.cu:240). */
int cumf_read_problem(const char *path, int pinned, cumf_problem *out);
/* Writes nnz 12-byte records (the inverse of read_problem; data/netflix/transform.cpp:37-42). */
int cumf_write_problem(const char *path, const cumf_problem *prob);
/* Allocates an empty problem of nnz records (pinned if asked). */
int cumf_alloc_problem(int64_t nnz, int pinned, cumf_problem *out);
int cumf_free_problem(cumf_problem *prob);

/* save_model (singleGPU/main.cpp:231-273): i32 fun=0, i32 m, i32 n, i32 k, f32 b, then
 * m*k f32 P, then n*k f32 Q.  Fails with CUMF_ERR_IO if the path cannot be written
 * (the reference prints and carries on with a NULL FILE*, main.cpp:242-245). */
int cumf_save_model(const cumf_model *model, const char *path);
/* mf_load_model (test/mf.cpp:3706-3777); also checks the file length. */
int cumf_load_model(const char *path, cumf_model *out);
int cumf_alloc_model(int32_t m, int32_t n, int32_t k, cumf_model *out);
int cumf_free_model(cumf_model *model);
/* Page-locked host buffers (pinned problems, models) are cached: cumf_free_problem and
 * cumf_free_model keep them (up to 2 GB in all, or CUMF_HOST_CACHE_MB megabytes from the
 * environment; 0 turns the cache off) for the next pinned allocation they fit,
 * because page-locking costs about 30 ms per GB and training calls repeat.  No counterpart
 * in the reference (which leaks its pinned buffers).  This call gives the cached buffers
 * back to the system; buffers still held by problems or models are not affected. */
int cumf_release_host_cache(void);

/* ---- rating text (data/netflix/transform.cpp) --------------------------------------- */

/* `./transform file_name` (data/netflix/transform.cpp:9-47) on the GPU: skips `header_lines`
 * lines the way fscanf(f, "%[^\n]\n") does (the reference skips 3, transform.cpp:31-33),
 * parses whitespace-separated "u v r" triples as fscanf("%d %d %f") does (transform.cpp:36)
 * and writes the 12-byte records to out_path (NULL: in_path + ".bin", transform.cpp:26).
 * Ratings are rounded to float exactly as strtof rounds.  Where fscanf would stop silently
 * or write a record with stale fields (a malformed token, a trailing partial triple), this
 * returns CUMF_ERR_FORMAT naming the byte offset; ids outside int32, hexadecimal floats and
 * ratings needing more than 19 significant digits to round are also rejected.
 * *n_records (may be NULL) receives the record count. */
int cumf_convert_text(const char *in_path, const char *out_path, int header_lines, int64_t *n_records);
/* The same parse into a problem (read_problem's result for the converted file, sgd.cu:190):
 * m = max u + 1, n = max v + 1; negative ids are rejected. */
int cumf_read_text_problem(const char *path, int header_lines, int pinned, cumf_problem *out);
/* Host helper: offset of the first data byte after `header_lines` header lines. */
int cumf_text_data_start(const char *text, int64_t len, int header_lines, int64_t *start);
/* Host text (preferably page-locked) -> host records, the text's copy, the parse and the
 * records' copy overlapped in chunks of about 64 MB.  Same rules as cumf_convert_text;
 * *n_records receives the count (out may be NULL with cap 0 to count only). */
int cumf_parse_text_host(const char *text, int64_t len, int header_lines, cumf_node *out, int64_t cap,
                         int64_t *n_records);
/* Device-level parse of text bytes [start, len) of d_text (16-byte aligned device memory)
 * into d_out.  *n_records receives the record count; with d_out == NULL only the count is
 * computed.  A d_out with cap < count fails with CUMF_ERR_ARG. Synchronises the stream. */
int cumf_dev_parse_text(const void *d_text, int64_t len, int64_t start, cumf_node *d_out, int64_t cap,
                        int64_t *n_records, void *stream);

/* ---- training --------------------------------------------------------------------- */
/* sgd_train (singleGPU/sgd.cu:638-690): stats -> shuffle ids -> grid -> scale -> init ->
 * batch-Hogwild epochs -> fp32 export, unscale, un-permute.  `va` may be NULL; when given,
 * and params.verbose_epochs is 1, the test RMSE is printed after each epoch.  `out` is
 * allocated by the call (free with cumf_free_model); `stats` may be NULL. */
int cumf_train(const cumf_problem *tr, const cumf_problem *va, const cumf_params *params,
               cumf_model *out, cumf_train_stats *stats);

/* calc_rmse (test/mf.cpp:3815-3839) on the GPU: sqrt(sum (r - <p_u,q_v>)^2 / nnz) with the
 * squared error rounded to fp32 and summed in fp64; ids outside the model or a NaN dot
 * predict model->b (mf.cpp:3794-3813). */
int cumf_rmse(const cumf_problem *te, const cumf_model *model, double *out);

/* Evaluation criteria of mf-predict -e (test/mf-predict.cpp:21-35; test/mf.cpp:3841-4044), on
 * the GPU: CUMF_EVAL_RMSE (0, same as cumf_rmse), MAE (1), GKL (2), LOGLOSS (5), ACCURACY (6),
 * ROW_MPR (10), COL_MPR (11), ROW_AUC (12), COL_AUC (13).  Positives for LOGLOSS, ACCURACY,
 * MPR and AUC are ratings r > 0, as in the reference.  MPR / AUC predict every (row, column)
 * of the rows that hold a positive (rows x max(te->n, model->n) dot products); test ids must
 * lie inside [0, max(te->m, model->m)) x [0, max(te->n, model->n)) (CUMF_ERR_RANGE otherwise;
 * the reference indexes out of bounds).  A set with no qualifying row gives NaN (0 / 0) as
 * the reference does.  Unknown criteria fail with CUMF_ERR_ARG ("unknown evaluation
 * criterion", mf-predict.cpp:64). */
enum {
    CUMF_EVAL_RMSE = 0, CUMF_EVAL_MAE = 1, CUMF_EVAL_GKL = 2, CUMF_EVAL_LOGLOSS = 5, CUMF_EVAL_ACC = 6,
    CUMF_EVAL_ROW_MPR = 10, CUMF_EVAL_COL_MPR = 11, CUMF_EVAL_ROW_AUC = 12, CUMF_EVAL_COL_AUC = 13
};
int cumf_evaluate(const cumf_problem *te, const cumf_model *model, int criterion, double *out);

/* ---- device-level entry points (caller-owned device memory) ----------------------- */
/* The learning-rate table lr[t] = (float)(alpha/(1+beta*t^1.5) + lrate), t < n
 * (singleGPU/sgd_kernel.cu:144-149), written to host memory. */
int cumf_lr_schedule(float alpha, float beta, float lrate, int n, float *out);
/* Per-worker batch budget ceil(nnz/(workers*128)) (singleGPU/sgd_kernel.cu:203). */
int64_t cumf_batches_per_worker(int64_t nnz, int num_workers);

/* random_init / init_feature (singleGPU/sgd.cu:497-546): every element of a rows x k
 * factor matrix is U(0,1] * (float)sqrt(1/k), rounded to the storage type.  The uniform
 * is a pure function of (seed, tag, element index). */
int cumf_dev_init_factors(void *d_factors, int64_t rows, int k, int precision,
                          uint64_t seed, uint32_t tag, void *stream);

/* sgd_update_k128 mode A / sgd_k128_kernel_hogwild_warp32_lrate
 * (singleGPU/sgd_kernel.cu:212-248, singleGPU/sgd_k128_kernel_hogwild_warp32.h:3-104):
 * runs epochs [first_epoch, first_epoch + n_epochs) of batch-Hogwild SGD in place on
 * d_P (m x k) and d_Q (n x k) over d_R (nnz records, ids already in range, ratings
 * scaled).  Each of `num_workers` workers does ceil(nnz/(num_workers*128)) batches per
 * epoch; a batch is 128 consecutive records from a uniformly drawn start (wrapping).
 * d_lr holds at least first_epoch+n_epochs learning rates (device memory).
 * d_status (device int, may be NULL) receives CUMF_ERR_RANGE if an index is out of range
 * (such a rating is skipped).  lanes = 0 picks the tuned default. */
int cumf_sgd_update(const cumf_node *d_R, int64_t nnz, void *d_P, int32_t m, void *d_Q,
                    int32_t n, int k, int precision, int num_workers, int lanes,
                    const float *d_lr, int first_epoch, int n_epochs, float lambda_p,
                    float lambda_q, uint64_t seed, int *d_status, void *stream);

/* cumf_sgd_update with explicit launch tuning (tuning may be NULL for the defaults). */
int cumf_sgd_update_tuned(const cumf_node *d_R, int64_t nnz, void *d_P, int32_t m, void *d_Q,
                          int32_t n, int k, int precision, int num_workers,
                          const cumf_tuning *tuning, const float *d_lr, int first_epoch,
                          int n_epochs, float lambda_p, float lambda_q, uint64_t seed,
                          int *d_status, void *stream);

/* ---- copies of the most-rated rows (no counterpart in the reference) -----------------
 * Batch-Hogwild workers that hold the same user or item row at the same moment serialise on
 * its cache lines; with skewed ids (Zipf item popularity) that bounds the epoch.  A row with
 * more than `per_copy` ratings gets min(max_copies, ceil(count / per_copy)) copies: the row
 * itself plus extra rows appended after the matrix's last row (rows m .. m_rows-1 of P,
 * n .. n_rows-1 of Q, in row order).  Rating i of such a row is assigned copy i mod copies.
 * The copies start equal (spread) and are averaged after each launch of epochs (merge: the
 * fp32 mean in copy order, rounded to nearest in the storage type, written to every copy),
 * so between launches every copy holds the row's value and exports read the row itself.
 * Use: plan on the shuffled, scaled ratings; allocate P and Q with m_rows and n_rows rows;
 * assign (rewrites the ratings' ids in place); init the first m / n rows; spread; then
 * cumf_sgd_update(..., m_rows, ..., n_rows, ...) and merge after every call.
 * cumf_train does this when params.hot_rows > 0 (off by default). */
typedef struct cumf_hot_rows cumf_hot_rows;

/* Ratings per copy for `concurrency` expected workers on one copy at a time: ceil(nnz *
 * concurrency / w), w = min(num_workers, resident workers of the update kernel for (k,
 * precision, lanes) on the current device), at least 4096.  0 (no copies) when
 * concurrency <= 0, num_workers < 2 or nnz == 0. */
int64_t cumf_hot_rows_per_copy(int64_t nnz, int32_t num_workers, int k, int precision, int lanes,
                               float concurrency);

/* Counts the ratings of every row and lays out the copies.  *out is freed with
 * cumf_hot_rows_free.  Ids outside [0, m) x [0, n) are not counted. */
int cumf_hot_rows_plan(const cumf_node *d_R, int64_t nnz, int32_t m, int32_t n, int64_t per_copy,
                       int32_t max_copies, cumf_hot_rows **out, void *stream);
/* Rows including the copies, and the number of rows that have copies (any may be NULL). */
int cumf_hot_rows_info(const cumf_hot_rows *plan, int32_t *m_rows, int32_t *n_rows, int32_t *hot_m,
                       int32_t *hot_n);
/* Copies the plan's tables out (host or device buffers; NULL skips one): per row of P and
 * of Q an int32 pair {copies, first extra row} (2*m and 2*n values; the second value of a
 * row without copies is the row itself), and the ascending lists of rows with copies (hot_m
 * and hot_n values).  Synchronous. */
int cumf_hot_rows_tables(const cumf_hot_rows *plan, int32_t *tab_m, int32_t *tab_n, int32_t *grp_m,
                         int32_t *grp_n);
/* Rewrites each rating of a row with copies to name its copy (i mod copies; copy 0 is the row). */
int cumf_hot_rows_assign(const cumf_hot_rows *plan, cumf_node *d_R, int64_t nnz, void *stream);
/* Copies each row with copies into its extra rows (bitwise). */
int cumf_hot_rows_spread(const cumf_hot_rows *plan, void *d_P, void *d_Q, int k, int precision,
                         void *stream);
/* Averages the copies of every row with copies and writes the mean to all of them. */
int cumf_hot_rows_merge(const cumf_hot_rows *plan, void *d_P, void *d_Q, int k, int precision,
                        void *stream);
int cumf_hot_rows_free(cumf_hot_rows *plan);

/* collect_data (singleGPU/sgd.cu:78-96) on the device: mean and population std of the
 * ratings, accumulated in fp64.  Results are written to host doubles. */
int cumf_dev_rating_stats(const cumf_node *d_R, int64_t nnz, double *mean, double *std_dev,
                          void *stream);

/* shuffle_problem + scale_problem (singleGPU/sgd.cu:126-134, 98-124, at u=v=1):
 * out[i] = {p_map[u], q_map[v], r * scale}; flags CUMF_ERR_RANGE in d_status when an id is
 * outside [0,m) x [0,n).  In-place (d_out == d_in) is allowed. */
int cumf_dev_shuffle_scale(const cumf_node *d_in, cumf_node *d_out, int64_t nnz,
                           const int32_t *d_p_map, int32_t m, const int32_t *d_q_map,
                           int32_t n, float scale, int *d_status, void *stream);

/* transform_half + scale_model + shuffle_model (singleGPU/sgd_kernel.cu:29-68,
 * sgd.cu:593-635): out[o] = float(in[map[o]]) * factor for every row o < rows (map may be
 * NULL for identity). */
int cumf_dev_export_factors(const void *d_in, int precision, const int32_t *d_map,
                            int64_t rows, int k, float factor, float *d_out, void *stream);

/* calc_rmse (test/mf.cpp:3815-3839) over device data: fp32 model P (m x k), Q (n x k).
 * The squared-error sum is reduced deterministically; *out_rmse is a host double. */
int cumf_dev_rmse(const cumf_node *d_R, int64_t nnz, const float *d_P, int32_t m,
                  const float *d_Q, int32_t n, int k, float b, double *out_rmse,
                  void *stream);

/* cumf_dev_rmse without any allocation.  No counterpart in the reference.  For callers that
 * cannot allocate device memory when they evaluate (inside a fixed memory pool or arena,
 * allocator hooks, out-of-memory handlers, code given only pre-sized buffers): the scratch
 * is a fixed __device__ array inside the library (16385 doubles, held by every GPU that loads
 * the library until exit), so nnz is limited to 134,217,728 ratings; larger calls return
 * CUMF_ERR_ARG.  All calls share that array: calls whose kernels overlap on the GPU race and
 * must be serialised by the caller.  The first call on each device (with that device
 * current) is its set-up: it looks up the array's address and loads the evaluator kernels,
 * which allocates under CUDA's lazy module loading; make it where allocation is still
 * possible (at start-up) and before any stream capture.  A call with nnz = 0 does only that
 * set-up.  Do not use it across a cudaDeviceReset (the cached address goes stale).  Same
 * inputs as cumf_dev_rmse; the result equals cumf_dev_rmse's within the rounding of the
 * double sum (different block split) and is identical from call to call. */
int cumf_dev_rmse_noalloc(const cumf_node *d_R, int64_t nnz, const float *d_P, int32_t m,
                          const float *d_Q, int32_t n, int k, float b, double *out_rmse,
                          void *stream);

/* Device SM count and the default worker count (52 warps-worth of workers per SM,
 * README.md:61, scaled for the lane width in use). */
int cumf_device_info(int gpu, int *sm_count, int *cc_major, int *cc_minor);
int cumf_default_workers(int sm_count, int k, int precision, int lanes);
/* Worker count for a problem of nnz ratings: 3 to 16 whole waves of resident workers (tail
 * balance), the count whose ceil(nnz / (W*128)) batches per worker overshoot nnz least, with
 * at least eight 128-record batches per worker; problems too small for three such waves get
 * nnz/1024 workers. */
int cumf_auto_workers(int64_t nnz, int sm_count, int k, int precision, int lanes);

/* glibc-compatible id shuffle used for bit-exact layout parity: fills map[0..size) with
 * the permutation that srand(seed); random_shuffle(identity) produces
 * (singleGPU/sgd.cu:39-53), without touching the process-wide rand() state. */
int cumf_random_map(uint32_t seed, int32_t size, int32_t *map);

/* grid_problem (singleGPU/sgd.cu:411-487): buckets R in place into ux*vy blocks in the
 * reference's exact order; grid_size receives ux*vy counts, u_seg/v_seg the segment sizes. */
int cumf_grid_problem(cumf_node *R, int64_t nnz, int32_t m, int32_t n, int ux, int vy,
                      int64_t *grid_size, int64_t *u_seg, int64_t *v_seg);

/* ---- warm-start MLP building blocks (no reference counterpart) -------------------- */
/* BF16 tensor-core GEMM (tcgen05, fp32 accumulation in tensor memory):
 *   out[M x N] = act(A[M x K] * B[N x K]^T + bias[N]),  A and B bf16 row-major,
 * act 0 = identity, 1 = GELU (tanh form); out is bf16 (out_f32 = 0) or fp32 with row stride
 * ldo; d_pre (may be NULL) receives the fp32 pre-activation.  K must be a multiple of 64;
 * M and N are arbitrary.  d_status (may be NULL) receives CUMF_ERR_TIMEOUT if a bounded
 * wait inside the kernel gives up. */
int cumf_tc_gemm(const void *d_A, const void *d_B, int M, int N, int K, const float *d_bias, int act,
                 void *d_out, int out_f32, int ldo, float *d_pre, int *d_status, void *stream);

/* User features for the warm start, from ratings and fp32 item factors Q (n x k): d_X
 * (m x (k+3)) = [sum_i (r_ui - mean_u) q_i / deg_u, log(1+deg_u)/4, (mean_u - 3)/2,
 * var_u/2]; users without ratings get zeros, ratings outside [0,m) x [0,n) are left out.
 * Below 2^32 ratings the sums run in each user's rating order (a stable sort by user), so
 * every call gives the same bits; the scratch comes from a pool of the library that keeps
 * up to 256 MB per device between calls. */
int cumf_user_features(const cumf_node *d_R, int64_t nnz, const float *d_Q, int32_t n, int k, int32_t m,
                       float *d_X, void *stream);

/* The warm-start MLP: d_in -> hidden (GELU) -> hidden (GELU) -> d_out, bf16 weights and
 * activations with fp32 accumulation on the tensor cores, fp32 master weights, Adam.
 * hidden and d_out must be multiples of 64.  The handle is opaque. */
int cumf_mlp_create(int d_in, int hidden, int d_out, uint64_t seed, void **mlp);
int cumf_mlp_destroy(void *mlp);
/* Parameters flattened as W1[hidden][d_in], b1, W2[hidden][hidden], b2, W3[d_out][hidden], b3. */
int64_t cumf_mlp_param_count(void *mlp);
/* which = 0: parameters, 1: gradients of the last cumf_mlp_loss_grad / training step. */
int cumf_mlp_get_params(void *mlp, float *host, int64_t count, int which);
int cumf_mlp_set_params(void *mlp, const float *host, int64_t count);
/* d_Y (rows x d_out, fp32) = MLP(d_X (rows x d_in, fp32)). */
int cumf_mlp_forward(void *mlp, const float *d_X, int64_t rows, float *d_Y, void *stream);
/* Mean-over-rows squared error against d_T and its gradients (kept in the handle). */
int cumf_mlp_loss_grad(void *mlp, const float *d_X, const float *d_T, int64_t rows, double *loss, void *stream);
/* Adam (0.9, 0.999) over shuffled mini-batches for `epochs` passes; *final_loss is the mean
 * loss of the last pass (0 for epochs == 0).  One training step is captured as a CUDA graph
 * and replayed per batch on a private stream ordered after `stream`; the next pass's
 * permutation is drawn on the host while the device runs the current one.  rows < 2^31;
 * batch > rows trains on whole passes.  Adam's step count carries over between calls. */
int cumf_mlp_train(void *mlp, const float *d_X, const float *d_T, int64_t rows, int epochs, int batch, float lr,
                   uint64_t seed, double *final_loss, void *stream);

/* cumf_train with a starting model and per-epoch evaluation (mode A only).  `init` (may be
 * NULL) gives starting fp32 factors in the model file's layout for the first init->m users and
 * init->n items (rows beyond them start from the usual random init); init->k must equal k.
 * init->pinned == 2 marks init->P and init->Q as device addresses (no host copy).
 * When `te` is given, epoch_rmse[e] receives the test RMSE after epoch e and epoch_ms[e] the
 * cumulative training time (CUDA events, evaluation excluded); either may be NULL. */
int cumf_train_ex(const cumf_problem *tr, const cumf_problem *te, const cumf_params *params,
                  const cumf_model *init, cumf_model *out, cumf_train_stats *stats, double *epoch_rmse,
                  double *epoch_ms);

/* Diagnostic (no reference counterpart): copy bandwidth (bytes read + written per second, GB/s)
 * of `passes` copies of a `bytes` buffer inside one launch, loads through L2 only.  With a
 * working set well inside L2 (e.g. 2 x 32 MB) it measures the L2-resident copy rate used as a
 * second roofline for the update kernel; with a large buffer, the HBM copy rate. */
int cumf_probe_copy_bandwidth(int64_t bytes, int passes, double *gbs, void *stream);

/* Self-test of the bounded waits (no reference counterpart): one tensor-core product whose
 * operand copies are deliberately not issued, so its stage wait runs out after about 2 s; the
 * kernel records CUMF_ERR_TIMEOUT in *status_out, drains and frees its tensor memory, and an
 * ordinary product on the same context is then checked.  *seconds (may be NULL) receives the
 * timed-out launch's duration.  Returns CUMF_OK when the context stayed usable. */
int cumf_selftest_wait_timeout(int *status_out, double *seconds);

/* ---- deterministic schedule (no reference counterpart) -------------------------------- */
/* Stratified SGD: ratings bucketed into a G x G grid of blocks (user group u mod G, item group
 * v mod G, stable order inside a block); an epoch runs the G strata in a seeded random order,
 * stratum s updating the blocks (a, (a + s) mod G), which share no user and no item, one worker per block, so the result is
 * the same on every run and equals the serial restatement bit for bit.  The per-rating
 * update is the batch-Hogwild kernel's (warp32.h:85-99; stochastic rounding keyed by the
 * rating's position in the sorted array). */
/* d_out (nnz records) and d_block_off (groups*groups + 1 offsets) receive the layout. */
int cumf_dev_strata_layout(const cumf_node *d_R, int64_t nnz, int groups, cumf_node *d_out,
                           unsigned long long *d_block_off, void *stream);
/* Epochs over the layout; h_lr is a host array indexed by epoch. */
int cumf_dev_strata_epochs(const cumf_node *d_S, const unsigned long long *d_block_off, int groups, void *d_P,
                           int32_t m, void *d_Q, int32_t n, int k, int precision, const float *h_lr,
                           int first_epoch, int n_epochs, float lambda_p, float lambda_q, uint64_t seed,
                           int *d_status, void *stream);

/* ---- checkpoint / resume (no reference counterpart) ---------------------------------- */
/* Periodic checkpoints of a mode-A run (u = v = 1).  The file holds the factors exactly as
 * training keeps them in HBM (permuted rows, scaled, storage precision), the number of
 * completed epochs and a fingerprint of the run (k, precision, workers, lanes, seed,
 * lambdas, learning-rate parameters, problem extent and a digest of the ratings).
 * Everything else (id maps, scaling, learning rates, sample draws) is recomputed from the
 * inputs, so a resumed run continues the same epoch sequence; with one worker (or any
 * deterministic configuration) it is bit-identical to an uninterrupted run that launches
 * the same epoch chunks.  Files are written to path + ".tmp" and renamed. */
typedef struct cumf_checkpoint {
    const char *path;      /* checkpoint file                                                */
    int32_t every;         /* write after every `every` completed epochs (0 = at the end)    */
    int32_t resume;        /* 1 = continue from `path` when it exists (it must match the run) */
    int32_t stop_after;    /* > 0: stop once this many epochs are complete and return the
                              model as it is then (an interrupted run); 0 = run all epochs   */
    int32_t reserved_[3];
} cumf_checkpoint;
/* cumf_train_ex with checkpoints: *epochs_done (may be NULL) receives the completed epoch
 * count.  A checkpoint that does not match the run or fails its digest is CUMF_ERR_FORMAT. */
int cumf_train_ckpt(const cumf_problem *tr, const cumf_problem *te, const cumf_params *params,
                    const cumf_checkpoint *ckpt, cumf_model *out, cumf_train_stats *stats, int32_t *epochs_done);

/* ---- batched factorizations (no reference counterpart) ------------------------------ */
/* One problem of a batch: device ratings with ids in range and ratings already scaled, fp16
 * factors P (m x k) and Q (n x k), k in {32, 64, 128}; num_workers 0 = set by the batch
 * tuning; d_lr has lr_len learning rates (epoch index < lr_len).  hot: copies of the
 * problem's most-rated rows (a cumf_hot_rows_plan of these m x n, cumf_hot_rows_assign
 * already applied to d_R, P and Q allocated with the plan's m_rows and n_rows rows and
 * spread), or NULL.  With any copies in the batch, cumf_batch_run launches one epoch at a
 * time and merges the copies after each (the launches stay in one graph). */
typedef struct cumf_batch_problem {
    const cumf_node *d_R;
    int64_t nnz;
    void *d_P;
    int32_t m;
    int32_t n;
    void *d_Q;
    int32_t k;
    int32_t num_workers;
    float lambda_p, lambda_q;
    uint64_t seed;
    const float *d_lr;
    int32_t lr_len;
    int32_t reserved_;
    const cumf_hot_rows *hot;
} cumf_batch_problem;

/* Schedule of a batched launch: workers per problem so each has about batches_target
 * 128-record batches per epoch (problems with num_workers > 0 keep theirs); task order
 * 0 = problem by problem, 1 = round robin over problems, 2 = largest problems first;
 * blocks_per_sm 1..4 of the persistent grid; lanes per worker 8, 16 or 32 (0 = 16; 32 needs
 * every problem's k >= 64), each lane moving k / lanes consecutive halves of a row. */
typedef struct cumf_batch_tuning {
    int32_t batches_target;
    int32_t order;
    int32_t blocks_per_sm;
    int32_t lanes;
    int32_t reserved_[4];
} cumf_batch_tuning;

/* Copies the problem descriptors (the device buffers stay the caller's). */
int cumf_batch_create(const cumf_batch_problem *probs, int count, void **batch);
int cumf_batch_destroy(void *batch);
int cumf_batch_set_tuning(void *batch, const cumf_batch_tuning *tuning);
int cumf_batch_get_info(void *batch, cumf_batch_tuning *tuning, int *tasks_per_epoch, int64_t *samples_per_epoch);
/* Epochs [first_epoch, first_epoch + n_epochs) of every problem in one persistent launch
 * (one launch per epoch, each followed by the merges, when a problem has row copies);
 * use_graph = 1 captures the launches (counter reset + kernel [+ merges]) in a CUDA graph on
 * first use and replays it while (first_epoch, n_epochs) and the tuning stay the same. */
int cumf_batch_run(void *batch, int first_epoch, int n_epochs, int use_graph, void *stream);
/* CUMF_ERR_RANGE if any launch met an out-of-range index (such ratings are skipped). */
int cumf_batch_status(void *batch, int *status);
/* Autotuner: times candidate schedules for one epoch each with a zero learning rate (factors
 * are left bit for bit unchanged) and keeps the fastest per sample: first lanes per worker
 * (8/16/32) x blocks per SM (3/4), then batch budget (4/8/16/32) x task order (0/1/2). */
int cumf_batch_autotune(void *batch, void *stream, cumf_batch_tuning *best, double *best_epoch_ms);

#ifdef __cplusplus
}
#endif

#endif /* CUMF_SGD_H_ */
