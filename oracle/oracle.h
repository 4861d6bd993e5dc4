/* oracle.h - CPU restatement of cuMF_SGD's batch-Hogwild SGD path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (cumf_sgd_gb300/, include/) links or
 * calls this code; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * use it, as the checker and as the timed CPU port.
 *
 * Each function names the reference lines it restates (paths inside the cuMF_SGD project).
 * Two things the reference leaves to runtime randomness are pinned here the same way the
 * GPU build pins them, so one worker replays the GPU's exact sample order:
 *   - batch starts: splitmix64 chain over (seed, epoch, worker, batch) -> mulhi(h, nnz)
 *     (the reference: curand_uniform * nnz, warp32.h:42-47);
 *   - factor init: U(0,1] from splitmix64(key ^ index) (the reference: curand, sgd.cu:512).
 * The id permutations use the real glibc srand()/rand() and a C restatement of libstdc++'s
 * random_shuffle, exactly as gen_random_map does (sgd.cu:39-53).
 */
#ifndef CUMF_ORACLE_H_
#define CUMF_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_node {
    int32_t u, v;
    float r;
} or_node;

/* storage kinds */
enum { OR_HALF = 0, OR_BF16 = 1, OR_FLOAT = 2 };
/* dot-product orders */
enum { OR_DOT_LANES = 0, /* G lanes, E contiguous elements each, butterfly (this build's kernel) */
       OR_DOT_REF = 1    /* 32 lanes, elements l+32j, shfl_down tree (warp32.h:62-83), k = 128 */ };
/* serialisation of the workers */
enum { OR_ORDER_WORKER_MAJOR = 0, OR_ORDER_ROUND_ROBIN = 1 };

/* numeric helpers */
uint16_t or_half_rn(float x);
float or_half_to_float(uint16_t h);
uint16_t or_bf16_rn(float x);
float or_bf16_to_float(uint16_t h);
float or_round_store(float x, int kind);          /* round to storage, back to float */
uint64_t or_splitmix64(uint64_t x);
uint32_t or_lowbias32(uint32_t x);
uint64_t or_batch_start(uint64_t seed, uint32_t epoch, uint32_t worker, uint32_t batch, uint64_t nnz);
uint64_t or_block_seed(uint64_t seed, int block);

/* collect_data (sgd.cu:78-96) */
void or_collect_data(const or_node *R, int64_t nnz, float *ave, float *std_dev);
/* gen_random_map (sgd.cu:39-53) with srand(seed) in place of srand(time(NULL)) */
void or_gen_random_map(uint32_t seed, int32_t size, int32_t *map);
/* the rand() calls of the mode B / C block shuffles that follow the maps */
void or_random_shuffle_int(int32_t *a, int64_t n);
/* shuffle_problem (sgd.cu:126-134) */
void or_shuffle_problem(or_node *R, int64_t nnz, const int32_t *pmap, const int32_t *qmap);
/* grid_problem (sgd.cu:411-487); grid_size has ux*vy entries */
void or_grid_problem(or_node *R, int64_t nnz, int32_t m, int32_t n, int ux, int vy,
                     int64_t *grid_size, int64_t *u_seg, int64_t *v_seg);
/* scale_problem (sgd.cu:98-124) */
void or_scale_problem(or_node *R, int64_t nnz, float scale, int ux, int vy, int64_t u_seg, int64_t v_seg);
/* dynamic_rate table (sgd_kernel.cu:144-149) */
void or_lr_table(float alpha, float beta, float lrate, int n, float *out);
/* init_feature: rows*k values rounded to storage kind (returned as floats) */
void or_init_factors(float *out, int64_t rows, int k, int kind, uint64_t seed, uint32_t tag);
/* scale_model (sgd.cu:593-606) */
void or_scale_model(float *P, int64_t rows, int k, float scale);
/* shuffle_model's inverse permutation by cycle following (sgd.cu:609-635); map is destroyed */
void or_shuffle_model(float *vec, int32_t *inv_map, int32_t size, int k);
/* calc_rmse / mf_predict (test/mf.cpp:3794-3839) */
double or_calc_rmse(const or_node *R, int64_t nnz, const float *P, int32_t m, const float *Q,
                    int32_t n, int k, float b);

/* Serial batch-Hogwild epochs (warp32.h:30-101 with the budget of sgd_kernel.cu:198-208).
 * P (m x k) and Q (n x k) hold storage-rounded values as floats and are updated in place.
 * sr = 1 applies this build's stochastic rounding with the same bits as the kernel. */
typedef struct or_sgd_args {
    const or_node *R;
    int64_t nnz;
    float *P;
    int32_t m;
    float *Q;
    int32_t n;
    int k;
    int kind;
    int sr;
    int num_workers;
    int lanes;           /* G for OR_DOT_LANES */
    int dot_order;
    int order;           /* worker serialisation */
    const float *lr;
    int first_epoch, n_epochs;
    float lambda_p, lambda_q;
    uint64_t seed;
    int64_t skipped;     /* out: records with an id out of range */
    int freeze_q;        /* 1: item rows are read but never written (user fold-in) */
} or_sgd_args;
void or_sgd_epochs(or_sgd_args *a);

/* Multi-threaded batch-Hogwild on the CPU (fp32 storage, OR_DOT_LANES order with G = 16):
 * workers are dealt round-robin to `threads` POSIX threads that update P and Q without
 * locks.  The timed CPU port of the path. */
void or_hogwild_threads(const or_node *R, int64_t nnz, float *P, int32_t m, float *Q, int32_t n,
                        int k, int num_workers, const float *lr, int first_epoch, int n_epochs,
                        float lambda_p, float lambda_q, uint64_t seed, int threads);

/* Full sgd_train (sgd.cu:638-690) for u = v = 1 (mode A), serial: outputs the fp32 model
 * (P: m x k, Q: n x k, already unscaled/un-permuted) and b.  R is not modified. */
typedef struct or_train_args {
    const or_node *R;
    int64_t nnz;
    int32_t m, n;
    int k;
    int kind, sr;
    int num_workers, lanes, dot_order, order;
    int num_iters;
    float lambda_p, lambda_q, alpha, beta, lrate;
    uint64_t seed;
    int u_grid, v_grid, x_grid, y_grid;   /* mode B / C when u_grid*v_grid > 1 */
    float *P_out;   /* m*k */
    float *Q_out;   /* n*k */
    float b_out;
    float ave, std_dev;
} or_train_args;
int or_train(or_train_args *a);

/* Serial FP64 SGD (the precision oracle): the same batch schedule as or_sgd_epochs, double
 * factors and arithmetic, no storage rounding. */
typedef struct or_sgd64_args {
    const or_node *R;
    int64_t nnz;
    double *P;
    int32_t m;
    double *Q;
    int32_t n;
    int k;
    int num_workers;
    int order;
    const double *lr;
    int first_epoch, n_epochs;
    double lambda_p, lambda_q;
    double rscale;       /* ratings are used as r * rscale (in double) */
    uint64_t seed;
} or_sgd64_args;
void or_sgd_epochs_f64(or_sgd64_args *a);
/* FP64 factor init: U(0,1] * sqrt(1/k) in double with the same uniforms as or_init_factors. */
void or_init_factors_f64(double *out, int64_t rows, int k, uint64_t seed, uint32_t tag);
/* The FP64 trainer's batches dealt to `threads` POSIX threads (Hogwild on the host). */
void or_sgd_epochs_f64_threads(or_sgd64_args *a, int threads);
/* RMSE of an FP64 model (double dot and error). */
double or_calc_rmse_f64(const or_node *R, int64_t nnz, const double *P, int32_t m, const double *Q,
                        int32_t n, int k, double b);

/* The deterministic stratified schedule (the library's strata.cu): records stably sorted by
 * block (u mod G) * G + (v mod G); epoch ep runs the strata in a seeded random order
 * (Fisher-Yates over 0 .. G-1 with splitmix64 draws), stratum s being the blocks
 * (a, (a + s) mod G) in any order (they share no rows), each block's records in order, with
 * the kernel's update (OR_DOT_LANES over `lanes`; stochastic rounding keyed by the record's
 * position in the sorted array).  Returns the number of records skipped as out of range. */
int64_t or_strata_epochs(const or_node *R, int64_t nnz, float *P, int32_t m, float *Q, int32_t n, int k, int kind,
                         int sr, int lanes, int G, const float *lr, int first_epoch, int n_epochs, float lambda_p,
                         float lambda_q, uint64_t seed);

/* data/netflix/transform.cpp:31-42 (the strict form the GPU converter implements): skips
 * `header_lines` lines as fscanf(f, "%[^\n]\n") does, then reads whitespace-separated
 * triples, u and v with strtol (the conversion behind %d) and r with strtof (behind %f).
 * Returns the record count, or -1 with *bad_offset = byte offset of the first token that is
 * not a complete decimal integer in int32 (u, v) or a complete decimal / inf / nan float (r),
 * or -2 when the token count is not a multiple of 3.  out may be NULL (count only). */
int64_t or_parse_text(const char *text, int64_t len, int header_lines, or_node *out, int64_t cap,
                      int64_t *bad_offset);

/* mf-predict's criteria (test/mf.cpp:3794-4044): 0 RMSE, 1 MAE, 2 GKL, 5 LOGLOSS, 6 ACCURACY,
 * 10 / 11 row- / column-wise MPR, 12 / 13 row- / column-wise AUC.  prob_m / prob_n are the
 * test problem's extent (mf_problem::m, n).  float predictions (sequential dot, NaN or
 * out-of-range ids -> b) and the reference's float / double mix.  Returns NAN for an
 * unknown criterion. */
double or_evaluate(const or_node *R, int64_t nnz, int32_t prob_m, int32_t prob_n, const float *P, int32_t m,
                   const float *Q, int32_t n, int k, float b, int criterion);

#ifdef __cplusplus
}
#endif
#endif
