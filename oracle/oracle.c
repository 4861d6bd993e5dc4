/* oracle.c - CPU restatement of cuMF_SGD's batch-Hogwild SGD path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Built with -ffp-contract=off so every fused
 * multiply-add below is an explicit fmaf() and nothing else is contracted.
 */
#include "oracle.h"

#include <ctype.h>
#include <errno.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---- fp16 / bf16 conversions (IEEE 754 binary16, round to nearest even) ------------- */

static uint32_t f2u(float x) { uint32_t u; memcpy(&u, &x, 4); return u; }
static float u2f(uint32_t u) { float x; memcpy(&x, &u, 4); return x; }

uint16_t or_half_rn(float x) {
    const uint32_t b = f2u(x);
    const uint16_t sign = (uint16_t)((b >> 16) & 0x8000u);
    const uint32_t ab = b & 0x7fffffffu;
    if (ab >= 0x7f800000u) /* inf or nan */
        return (uint16_t)(sign | 0x7c00u | (ab > 0x7f800000u ? 0x200u | ((ab >> 13) & 0x3ffu) : 0));
    if (ab >= 0x477ff000u) /* rounds to >= 65520 -> inf */
        return (uint16_t)(sign | 0x7c00u);
    const int e = (int)(ab >> 23) - 127;
    if (e >= -14) { /* normal half */
        uint32_t mant = ab & 0x7fffffu;
        uint32_t h = ((uint32_t)(e + 15) << 10) | (mant >> 13);
        const uint32_t rest = mant & 0x1fffu;
        if (rest > 0x1000u || (rest == 0x1000u && (h & 1u))) h += 1; /* carry may bump exponent */
        return (uint16_t)(sign | h);
    }
    /* subnormal half: value = m * 2^-24 */
    if (e < -25) return sign; /* below half of the smallest subnormal */
    const uint32_t mant = (ab & 0x7fffffu) | 0x800000u; /* 24-bit significand, value mant*2^(e-23) */
    const int shift = -e - 1;                            /* 2^(e-23) / 2^-24 = 2^(e+1) */
    uint32_t h = mant >> shift;
    const uint32_t rest = mant & ((1u << shift) - 1u);
    const uint32_t halfway = 1u << (shift - 1);
    if (rest > halfway || (rest == halfway && (h & 1u))) h += 1;
    return (uint16_t)(sign | h);
}

float or_half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t exp = (h >> 10) & 0x1fu, man = h & 0x3ffu;
    if (exp == 0) {
        const float v = (float)man * (1.0f / 16777216.0f); /* man * 2^-24, exact */
        return sign ? -v : v;
    }
    if (exp == 0x1f) return u2f(sign | 0x7f800000u | (man << 13));
    return u2f(sign | ((exp + 112u) << 23) | (man << 13));
}

uint16_t or_bf16_rn(float x) {
    const uint32_t b = f2u(x);
    if ((b & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((b >> 16) | 0x40u); /* quiet nan */
    const uint32_t lsb = (b >> 16) & 1u;
    return (uint16_t)((b + 0x7fffu + lsb) >> 16);
}

float or_bf16_to_float(uint16_t h) { return u2f((uint32_t)h << 16); }

float or_round_store(float x, int kind) {
    if (kind == OR_HALF) return or_half_to_float(or_half_rn(x));
    if (kind == OR_BF16) return or_bf16_to_float(or_bf16_rn(x));
    return x;
}

/* neighbouring halves of x: lo <= x <= hi */
static void half_bracket(float x, float *lo, float *hi) {
    const uint16_t h = or_half_rn(x);
    const float f = or_half_to_float(h);
    if (f == x || isnan(x) || isinf(f)) { *lo = *hi = f; return; }
    /* step one half-ulp pattern towards x */
    uint16_t other;
    const int up = f < x;
    if ((h & 0x7fffu) == 0) other = up ? 0x0001u : 0x8001u;
    else if (((h & 0x8000u) == 0) == up) other = (uint16_t)(h + 1);
    else other = (uint16_t)(h - 1);
    const float g = or_half_to_float(other);
    if (up) { *lo = f; *hi = g; } else { *lo = g; *hi = f; }
}

/* Stochastic rounding with 16 random bits, as the kernel does. */
static float half_sr(float x, uint32_t r16) {
    float lo, hi;
    half_bracket(x, &lo, &hi);
    if (lo == hi) return lo;
    const float u = (float)r16 * (1.0f / 65536.0f);
    return (x - lo > u * (hi - lo)) ? hi : lo;
}

static float bf16_sr(float x, uint32_t r16) {
    const uint32_t b = f2u(x);
    if ((b & 0x7f800000u) == 0x7f800000u) return or_bf16_to_float(or_bf16_rn(x));
    return u2f(((b + r16) >> 16) << 16);
}

/* ---- counter-based draws (SplitMix64, Steele/Lea/Flood 2014; lowbias32, Wellons 2018) -- */

uint64_t or_splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint32_t or_lowbias32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

uint64_t or_batch_start(uint64_t seed, uint32_t epoch, uint32_t worker, uint32_t batch, uint64_t nnz) {
    uint64_t h = or_splitmix64(seed ^ (0x5341ull << 48));
    h = or_splitmix64(h + epoch);
    h = or_splitmix64(h + worker);
    h = or_splitmix64(h + batch);
    return (uint64_t)(((unsigned __int128)h * nnz) >> 64);
}

uint64_t or_block_seed(uint64_t seed, int block) { return seed + (uint64_t)block * 0x9E3779B97F4A7C15ull; }

static float init_uniform(uint64_t key, uint64_t index) {
    const uint64_t h = or_splitmix64(key ^ index);
    return (float)((h >> 40) + 1) * (1.0f / 16777216.0f);
}

/* ---- data preparation --------------------------------------------------------------- */

void or_collect_data(const or_node *R, int64_t nnz, float *ave, float *std_dev) {
    double ex = 0, ex2 = 0;
    for (int64_t i = 0; i < nnz; i++) {
        const float r = R[i].r;
        ex += (double)r;
        ex2 += (double)r * r;
    }
    ex = ex / (double)nnz;
    ex2 = ex2 / (double)nnz;
    *ave = (float)ex;
    *std_dev = (float)sqrt(ex2 - ex * ex);
}

/* libstdc++ random_shuffle(first, last): j = rand() % (i + 1) for i = 1 .. n-1 */
void or_random_shuffle_int(int32_t *a, int64_t n) {
    for (int64_t i = 1; i < n; i++) {
        const int64_t j = (int64_t)rand() % (i + 1);
        if (i != j) {
            const int32_t t = a[i];
            a[i] = a[j];
            a[j] = t;
        }
    }
}

void or_gen_random_map(uint32_t seed, int32_t size, int32_t *map) {
    srand(seed);
    for (int32_t i = 0; i < size; i++) map[i] = i;
    or_random_shuffle_int(map, size);
}

void or_shuffle_problem(or_node *R, int64_t nnz, const int32_t *pmap, const int32_t *qmap) {
    for (int64_t i = 0; i < nnz; i++) {
        R[i].u = pmap[R[i].u];
        R[i].v = qmap[R[i].v];
    }
}

void or_grid_problem(or_node *R, int64_t nnz, int32_t m, int32_t n, int ux, int vy,
                     int64_t *grid_size, int64_t *u_seg_out, int64_t *v_seg_out) {
    const int64_t u_seg = ux == 1 ? m : (int64_t)ceil((double)m / ux);
    const int64_t v_seg = vy == 1 ? n : (int64_t)ceil((double)n / vy);
    *u_seg_out = u_seg;
    *v_seg_out = v_seg;
    const int G = ux * vy;
    memset(grid_size, 0, sizeof(int64_t) * G);
    for (int64_t i = 0; i < nnz; i++) grid_size[(R[i].u / u_seg) * vy + R[i].v / v_seg]++;
    int64_t *ends = (int64_t *)malloc(sizeof(int64_t) * (G + 1));
    int64_t *pivots = (int64_t *)malloc(sizeof(int64_t) * G);
    ends[0] = 0;
    for (int g = 0; g < G; g++) ends[g + 1] = ends[g] + grid_size[g];
    for (int g = 0; g < G; g++) pivots[g] = ends[g];
    for (int g = 0; g < G; g++) {
        int64_t pivot = pivots[g];
        while (pivot != ends[g + 1]) {
            const int c = (int)((R[pivot].u / u_seg) * vy + R[pivot].v / v_seg);
            if (c == g) { pivot++; continue; }
            const or_node t = R[pivot];
            R[pivot] = R[pivots[c]];
            R[pivots[c]] = t;
            pivots[c]++;
        }
    }
    free(ends);
    free(pivots);
}

void or_scale_problem(or_node *R, int64_t nnz, float scale, int ux, int vy, int64_t u_seg, int64_t v_seg) {
    for (int64_t i = 0; i < nnz; i++) {
        R[i].r = R[i].r * scale;
        if (ux * vy != 1) {
            int64_t u = R[i].u, v = R[i].v;
            while (u >= u_seg) u -= u_seg;
            while (v >= v_seg) v -= v_seg;
            R[i].u = (int32_t)u;
            R[i].v = (int32_t)v;
        }
    }
}

void or_lr_table(float alpha, float beta, float lrate, int n, float *out) {
    for (int i = 0; i < n; i++) out[i] = (float)(alpha / (1 + beta * pow((double)i, 1.5)) + lrate);
}

void or_init_factors(float *out, int64_t rows, int k, int kind, uint64_t seed, uint32_t tag) {
    const uint64_t key = or_splitmix64(or_splitmix64(seed) + tag);
    const float scale = (float)sqrt(1.0 / (double)k);
    const int64_t count = rows * (int64_t)k;
    for (int64_t i = 0; i < count; i++) out[i] = or_round_store(init_uniform(key, (uint64_t)i) * scale, kind);
}

void or_scale_model(float *P, int64_t rows, int k, float scale) {
    const float f = (float)sqrt(scale);
    for (int64_t i = 0; i < rows * (int64_t)k; i++) P[i] = P[i] * f;
}

void or_shuffle_model(float *vec, int32_t *map, int32_t size, int k) {
    for (int32_t pivot = 0; pivot < size;) {
        if (pivot == map[pivot]) { ++pivot; continue; }
        const int32_t next = map[pivot];
        for (int d = 0; d < k; d++) {
            const float t = vec[(int64_t)pivot * k + d];
            vec[(int64_t)pivot * k + d] = vec[(int64_t)next * k + d];
            vec[(int64_t)next * k + d] = t;
        }
        map[pivot] = map[next];
        map[next] = next;
    }
}

double or_calc_rmse(const or_node *R, int64_t nnz, const float *P, int32_t m, const float *Q,
                    int32_t n, int k, float b) {
    if (nnz == 0) return 0;
    double loss = 0;
    for (int64_t i = 0; i < nnz; i++) {
        const int32_t u = R[i].u, v = R[i].v;
        float z;
        if (u < 0 || u >= m || v < 0 || v >= n) {
            z = b;
        } else {
            const float *p = P + (int64_t)u * k, *q = Q + (int64_t)v * k;
            z = 0.0f; /* std::inner_product in index order */
            for (int d = 0; d < k; d++) z = z + p[d] * q[d];
            if (isnan(z)) z = b;
        }
        const float e = R[i].r - z;
        loss += e * e;
    }
    return sqrt(loss / nnz);
}

/* ---- the update ---------------------------------------------------------------------- */

static float dot_lanes(const float *p, const float *q, int k, int G) {
    float s[32];
    const int E = k / G;
    for (int l = 0; l < G; l++) {
        float acc = 0.0f;
        for (int e = 0; e < E; e++) acc = fmaf(p[l * E + e], q[l * E + e], acc);
        s[l] = acc;
    }
    for (int o = G / 2; o >= 1; o >>= 1) {
        float t[32];
        for (int l = 0; l < G; l++) t[l] = s[l] + s[l ^ o];
        memcpy(s, t, sizeof(float) * G);
    }
    return s[0];
}

/* warp32.h:62-83: lane l holds l, l+32, l+64, l+96; partial (contracted by nvcc into an
 * fma chain), then shfl_down 16, 8, 4, 2, 1 and the value of lane 0. */
static float dot_ref(const float *p, const float *q) {
    float s[32];
    for (int l = 0; l < 32; l++) {
        float acc = p[l] * q[l];
        acc = fmaf(p[l + 32], q[l + 32], acc);
        acc = fmaf(p[l + 64], q[l + 64], acc);
        acc = fmaf(p[l + 96], q[l + 96], acc);
        s[l] = acc;
    }
    for (int o = 16; o >= 1; o >>= 1)
        for (int l = 0; l < o; l++) s[l] = s[l] + s[l + o];
    return s[0];
}

/* One SGD update of rows p, q with rating r (warp32.h:85-99), in the kernel's fma order. */
static void update_rows(float *p, float *q, int k, float r, float lr, float lp, float lq, int kind,
                        int sr, uint32_t key, int G, int dot_order, int freeze_q) {
    const float s = dot_order == OR_DOT_REF ? dot_ref(p, q) : dot_lanes(p, q, k, G);
    const float err = r - s;
    for (int d = 0; d < k; d++) {
        const float pp = p[d], qq = q[d];
        const float pn = fmaf(lr, fmaf(err, qq, -(lp * pp)), pp);
        const float qn = fmaf(lr, fmaf(err, pp, -(lq * qq)), qq);
        if (sr && kind != OR_FLOAT) {
            const uint32_t pair = (uint32_t)(d / 2) * 2u;
            const uint32_t bp = or_lowbias32(key + pair), bq = or_lowbias32(key + pair + 1u);
            const uint32_t rp = (d & 1) ? (bp >> 16) : (bp & 0xffffu);
            const uint32_t rq = (d & 1) ? (bq >> 16) : (bq & 0xffffu);
            p[d] = kind == OR_HALF ? half_sr(pn, rp) : bf16_sr(pn, rp);
            if (!freeze_q) q[d] = kind == OR_HALF ? half_sr(qn, rq) : bf16_sr(qn, rq);
        } else {
            p[d] = or_round_store(pn, kind);
            if (!freeze_q) q[d] = or_round_store(qn, kind);
        }
    }
}

static void run_batch(or_sgd_args *a, int ep, int w, int64_t b, int64_t batches, float lr, uint32_t round_key) {
    const uint64_t start = or_batch_start(a->seed, (uint32_t)ep, (uint32_t)w, (uint32_t)b, (uint64_t)a->nnz);
    for (int i = 0; i < 128; i++) {
        const uint64_t rec = (start + (uint64_t)i) % (uint64_t)a->nnz;
        const or_node x = a->R[rec];
        if ((uint32_t)x.u >= (uint32_t)a->m || (uint32_t)x.v >= (uint32_t)a->n) {
            a->skipped++;
            continue;
        }
        uint32_t key = 0;
        if (a->sr) {
            const uint32_t sample = (uint32_t)w * (uint32_t)(batches * 128) + (uint32_t)(b * 128 + i);
            key = round_key ^ or_lowbias32(sample);
        }
        update_rows(a->P + (int64_t)x.u * a->k, a->Q + (int64_t)x.v * a->k, a->k, x.r, lr, a->lambda_p,
                    a->lambda_q, a->kind, a->sr, key, a->lanes, a->dot_order, a->freeze_q);
    }
}

void or_sgd_epochs(or_sgd_args *a) {
    a->skipped = 0;
    if (a->nnz <= 0 || a->num_workers <= 0) return;
    const int64_t per = (int64_t)a->num_workers * 128;
    const int64_t batches = (a->nnz + per - 1) / per;
    for (int ep = a->first_epoch; ep < a->first_epoch + a->n_epochs; ep++) {
        const float lr = a->lr[ep];
        const uint32_t round_key = (uint32_t)(or_splitmix64(a->seed ^ (0x5352ull << 48)) + (uint64_t)ep);
        if (a->order == OR_ORDER_WORKER_MAJOR) {
            for (int w = 0; w < a->num_workers; w++)
                for (int64_t b = 0; b < batches; b++) run_batch(a, ep, w, b, batches, lr, round_key);
        } else {
            for (int64_t b = 0; b < batches; b++)
                for (int w = 0; w < a->num_workers; w++) run_batch(a, ep, w, b, batches, lr, round_key);
        }
    }
}

/* ---- threaded CPU port ------------------------------------------------------------------ */

typedef struct {
    or_sgd_args base;
    int tid, threads;
} hog_arg;

static void *hog_thread(void *p) {
    hog_arg *h = (hog_arg *)p;
    or_sgd_args *a = &h->base;
    const int64_t per = (int64_t)a->num_workers * 128;
    const int64_t batches = (a->nnz + per - 1) / per;
    for (int ep = a->first_epoch; ep < a->first_epoch + a->n_epochs; ep++)
        for (int64_t b = 0; b < batches; b++)
            for (int w = h->tid; w < a->num_workers; w += h->threads) run_batch(a, ep, w, b, batches, a->lr[ep], 0);
    return NULL;
}

void or_hogwild_threads(const or_node *R, int64_t nnz, float *P, int32_t m, float *Q, int32_t n,
                        int k, int num_workers, const float *lr, int first_epoch, int n_epochs,
                        float lambda_p, float lambda_q, uint64_t seed, int threads) {
    if (threads < 1) threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    hog_arg *args = (hog_arg *)calloc(threads, sizeof(hog_arg));
    for (int t = 0; t < threads; t++) {
        or_sgd_args *a = &args[t].base;
        a->R = R; a->nnz = nnz; a->P = P; a->m = m; a->Q = Q; a->n = n; a->k = k;
        a->kind = OR_FLOAT; a->sr = 0; a->num_workers = num_workers; a->lanes = 16;
        a->dot_order = OR_DOT_LANES; a->lr = lr; a->first_epoch = first_epoch; a->n_epochs = n_epochs;
        a->lambda_p = lambda_p; a->lambda_q = lambda_q; a->seed = seed;
        args[t].tid = t;
        args[t].threads = threads;
        pthread_create(&th[t], NULL, hog_thread, &args[t]);
    }
    for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
    free(th);
    free(args);
}

/* ---- sgd_train ----------------------------------------------------------------------------- */

static void shuffle_block_order_b(int32_t *u_ids, int ug, int32_t *v_ids, int vg, int u_ite) {
    (void)u_ids; (void)ug; (void)u_ite;
    or_random_shuffle_int(v_ids, vg);
}

int or_train(or_train_args *a) {
    const int64_t nnz = a->nnz;
    const int k = a->k;
    or_node *R = (or_node *)malloc(sizeof(or_node) * (nnz ? nnz : 1));
    memcpy(R, a->R, sizeof(or_node) * nnz);
    float ave, std_dev;
    or_collect_data(R, nnz, &ave, &std_dev);
    const float scale = std_dev > 1e-4f ? std_dev : 1e-4f;
    a->ave = ave;
    a->std_dev = std_dev;

    int32_t *pmap = (int32_t *)malloc(sizeof(int32_t) * a->m);
    int32_t *qmap = (int32_t *)malloc(sizeof(int32_t) * a->n);
    or_gen_random_map((uint32_t)a->seed, a->m, pmap);
    or_gen_random_map((uint32_t)a->seed, a->n, qmap); /* rand() stream continues from here */
    or_shuffle_problem(R, nnz, pmap, qmap);

    const int ug = a->u_grid, vg = a->v_grid;
    const int xg = ug * vg == 1 ? 1 : a->x_grid, yg = ug * vg == 1 ? 1 : a->y_grid;
    const int ux = ug * xg, vy = vg * yg;
    int64_t *grid_size = (int64_t *)malloc(sizeof(int64_t) * ux * vy);
    int64_t u_seg, v_seg;
    or_grid_problem(R, nnz, a->m, a->n, ux, vy, grid_size, &u_seg, &v_seg);
    or_scale_problem(R, nnz, (float)(1.0 / scale), ux, vy, u_seg, v_seg);
    const float lambda_p = a->lambda_p / scale, lambda_q = a->lambda_q / scale;

    const int64_t prow = (int64_t)ux * u_seg, qrow = (int64_t)vy * v_seg;
    float *P = (float *)malloc(sizeof(float) * prow * k);
    float *Q = (float *)malloc(sizeof(float) * qrow * k);
    or_init_factors(P, prow, k, a->kind, a->seed, 1);
    or_init_factors(Q, qrow, k, a->kind, a->seed, 2);

    const int nlr = a->num_iters + 4;
    float *lr = (float *)malloc(sizeof(float) * nlr);
    or_lr_table(a->alpha, a->beta, a->lrate, nlr, lr);

    int64_t *begin = (int64_t *)malloc(sizeof(int64_t) * (ux * vy + 1));
    begin[0] = 0;
    for (int g = 0; g < ux * vy; g++) begin[g + 1] = begin[g] + grid_size[g];

    or_sgd_args s;
    memset(&s, 0, sizeof(s));
    s.k = k; s.kind = a->kind; s.sr = a->sr; s.num_workers = a->num_workers; s.lanes = a->lanes;
    s.dot_order = a->dot_order; s.order = a->order; s.lr = lr; s.lambda_p = lambda_p; s.lambda_q = lambda_q;

    if (ux * vy == 1) {
        s.R = R; s.nnz = nnz; s.P = P; s.m = a->m; s.Q = Q; s.n = a->n;
        s.first_epoch = 0; s.n_epochs = a->num_iters; s.seed = a->seed;
        or_sgd_epochs(&s);
    } else {
        /* mode B (sgd_kernel.cu:249-372) and mode C (:373-690) block schedules, one block at
         * a time; in mode C the x*y sub-blocks of a u*v block run in natural order because
         * global_*_list is indexed by the sub-block's own id (:440-448). */
        int32_t *u_ids = (int32_t *)malloc(sizeof(int32_t) * ug);
        int32_t *v_ids = (int32_t *)malloc(sizeof(int32_t) * vg);
        int32_t *uv_ids = (int32_t *)malloc(sizeof(int32_t) * ug * vg);
        int32_t *x_ids = (int32_t *)malloc(sizeof(int32_t) * xg);
        int32_t *y_ids = (int32_t *)malloc(sizeof(int32_t) * yg);
        int32_t *xy_ids = (int32_t *)malloc(sizeof(int32_t) * xg * yg);
        for (int i = 0; i < ug; i++) u_ids[i] = i;
        for (int i = 0; i < vg; i++) v_ids[i] = i;
        for (int i = 0; i < ug * vg; i++) uv_ids[i] = i;
        for (int i = 0; i < xg; i++) x_ids[i] = i;
        for (int i = 0; i < yg; i++) y_ids[i] = i;
        for (int i = 0; i < xg * yg; i++) xy_ids[i] = i;
        const int mode_c = xg * yg > 1;
        for (int iter = 0; iter < a->num_iters; iter++) {
            if (mode_c) or_random_shuffle_int(uv_ids, ug * vg);
            or_random_shuffle_int(u_ids, ug);
            for (int u_ite = 0; u_ite < ug; u_ite++) {
                if (!mode_c) shuffle_block_order_b(u_ids, ug, v_ids, vg, u_ite);
                for (int v_ite = 0; v_ite < vg; v_ite++) {
                    int cu, cv;
                    if (mode_c) {
                        cu = uv_ids[u_ite * vg + v_ite] / vg;
                        cv = uv_ids[u_ite * vg + v_ite] % vg;
                        or_random_shuffle_int(x_ids, xg);
                        or_random_shuffle_int(xy_ids, xg * yg);
                        for (int lx = 0; lx < xg; lx++) or_random_shuffle_int(y_ids, yg);
                    } else {
                        cu = u_ids[u_ite];
                        cv = v_ids[v_ite];
                    }
                    for (int sub = 0; sub < xg * yg; sub++) {
                        const int gx = cu * xg + sub / yg, gy = cv * yg + sub % yg;
                        const int g = gx * vy + gy;
                        s.R = R + begin[g]; s.nnz = grid_size[g];
                        s.P = P + (int64_t)gx * u_seg * k; s.m = (int32_t)u_seg;
                        s.Q = Q + (int64_t)gy * v_seg * k; s.n = (int32_t)v_seg;
                        s.first_epoch = iter; s.n_epochs = 1; s.seed = or_block_seed(a->seed, g);
                        or_sgd_epochs(&s);
                    }
                }
            }
        }
        free(u_ids); free(v_ids); free(uv_ids); free(x_ids); free(y_ids); free(xy_ids);
    }

    or_scale_model(P, prow, k, scale);
    or_scale_model(Q, qrow, k, scale);
    int32_t *inv_p = (int32_t *)malloc(sizeof(int32_t) * a->m);
    int32_t *inv_q = (int32_t *)malloc(sizeof(int32_t) * a->n);
    for (int32_t i = 0; i < a->m; i++) inv_p[pmap[i]] = i;
    for (int32_t i = 0; i < a->n; i++) inv_q[qmap[i]] = i;
    or_shuffle_model(P, inv_p, a->m, k);
    or_shuffle_model(Q, inv_q, a->n, k);
    memcpy(a->P_out, P, sizeof(float) * (size_t)a->m * k);
    memcpy(a->Q_out, Q, sizeof(float) * (size_t)a->n * k);
    a->b_out = ave / std_dev;

    free(R); free(pmap); free(qmap); free(grid_size); free(P); free(Q); free(lr); free(begin);
    free(inv_p); free(inv_q);
    return 0;
}

/* ---- FP64 precision oracle ---------------------------------------------------------------- */

void or_init_factors_f64(double *out, int64_t rows, int k, uint64_t seed, uint32_t tag) {
    const uint64_t key = or_splitmix64(or_splitmix64(seed) + tag);
    const double scale = sqrt(1.0 / (double)k);
    const int64_t count = rows * (int64_t)k;
    for (int64_t i = 0; i < count; i++) out[i] = (double)init_uniform(key, (uint64_t)i) * scale;
}

static void run_batch_f64(or_sgd64_args *a, int ep, int w, int64_t b, double lr) {
    const uint64_t start = or_batch_start(a->seed, (uint32_t)ep, (uint32_t)w, (uint32_t)b, (uint64_t)a->nnz);
    const int k = a->k;
    for (int i = 0; i < 128; i++) {
        const or_node x = a->R[(start + (uint64_t)i) % (uint64_t)a->nnz];
        if ((uint32_t)x.u >= (uint32_t)a->m || (uint32_t)x.v >= (uint32_t)a->n) continue;
        double *p = a->P + (int64_t)x.u * k, *q = a->Q + (int64_t)x.v * k;
        double dot = 0;
        for (int d = 0; d < k; d++) dot += p[d] * q[d];
        const double err = (double)x.r * a->rscale - dot;
        for (int d = 0; d < k; d++) {
            const double pp = p[d], qq = q[d];
            p[d] = pp + lr * (err * qq - a->lambda_p * pp);
            q[d] = qq + lr * (err * pp - a->lambda_q * qq);
        }
    }
}

void or_sgd_epochs_f64(or_sgd64_args *a) {
    if (a->nnz <= 0 || a->num_workers <= 0) return;
    const int64_t per = (int64_t)a->num_workers * 128;
    const int64_t batches = (a->nnz + per - 1) / per;
    for (int ep = a->first_epoch; ep < a->first_epoch + a->n_epochs; ep++) {
        const double lr = a->lr[ep];
        if (a->order == OR_ORDER_WORKER_MAJOR) {
            for (int w = 0; w < a->num_workers; w++)
                for (int64_t b = 0; b < batches; b++) run_batch_f64(a, ep, w, b, lr);
        } else {
            for (int64_t b = 0; b < batches; b++)
                for (int w = 0; w < a->num_workers; w++) run_batch_f64(a, ep, w, b, lr);
        }
    }
}

double or_calc_rmse_f64(const or_node *R, int64_t nnz, const double *P, int32_t m, const double *Q,
                        int32_t n, int k, double b) {
    if (nnz == 0) return 0;
    double loss = 0;
    for (int64_t i = 0; i < nnz; i++) {
        const int32_t u = R[i].u, v = R[i].v;
        double z = b;
        if (u >= 0 && u < m && v >= 0 && v < n) {
            const double *p = P + (int64_t)u * k, *q = Q + (int64_t)v * k;
            z = 0;
            for (int d = 0; d < k; d++) z += p[d] * q[d];
            if (isnan(z)) z = b;
        }
        const double e = (double)R[i].r - z;
        loss += e * e;
    }
    return sqrt(loss / (double)nnz);
}

typedef struct {
    or_sgd64_args *a;
    int tid, threads;
} f64_thread_arg;

static void *f64_thread(void *p) {
    f64_thread_arg *t = (f64_thread_arg *)p;
    or_sgd64_args *a = t->a;
    const int64_t per = (int64_t)a->num_workers * 128;
    const int64_t batches = (a->nnz + per - 1) / per;
    for (int ep = a->first_epoch; ep < a->first_epoch + a->n_epochs; ep++)
        for (int64_t b = 0; b < batches; b++)
            for (int w = t->tid; w < a->num_workers; w += t->threads) run_batch_f64(a, ep, w, b, a->lr[ep]);
    return NULL;
}

void or_sgd_epochs_f64_threads(or_sgd64_args *a, int threads) {
    if (a->nnz <= 0 || a->num_workers <= 0) return;
    if (threads < 1) threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    f64_thread_arg *args = (f64_thread_arg *)malloc(sizeof(f64_thread_arg) * threads);
    for (int t = 0; t < threads; t++) {
        args[t].a = a;
        args[t].tid = t;
        args[t].threads = threads;
        pthread_create(&th[t], NULL, f64_thread, &args[t]);
    }
    for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
    free(th);
    free(args);
}


/* ---- rating text (data/netflix/transform.cpp:31-42) ------------------------------------- */

static int or_space(unsigned char c) { return c == ' ' || (c >= '\t' && c <= '\r'); }

int64_t or_parse_text(const char *text, int64_t len, int header_lines, or_node *out, int64_t cap,
                      int64_t *bad_offset) {
    const unsigned char *p = (const unsigned char *)text;
    int64_t i = 0, ntok = 0;
    /* fscanf(file_in, "%[^\n]\n", line) x header_lines (transform.cpp:31-33): the scanset
     * needs at least one character, so an empty line (or the end) stops this and later calls. */
    for (int h = 0; h < header_lines; ++h) {
        if (i >= len || p[i] == '\n') break;
        while (i < len && p[i] != '\n') ++i;
        while (i < len && or_space(p[i])) ++i;
    }
    char tok[1100];
    or_node rec = {0, 0, 0.f};
    while (1) {
        while (i < len && or_space(p[i])) ++i;
        if (i >= len) break;
        const int64_t t0 = i;
        while (i < len && !or_space(p[i])) ++i;
        const int64_t tl = i - t0;
        if (tl >= (int64_t)sizeof(tok)) {
            *bad_offset = t0;
            return -1;
        }
        memcpy(tok, p + t0, (size_t)tl);
        tok[tl] = 0;
        const int field = (int)(ntok % 3);
        char *end = NULL;
        errno = 0;
        if (field < 2) {
            /* %d: optional sign and decimal digits only */
            const char *q = tok + ((tok[0] == '+' || tok[0] == '-') ? 1 : 0);
            int ok = *q != 0;
            for (const char *c = q; *c; ++c) ok &= isdigit((unsigned char)*c) != 0;
            long long v = ok ? strtoll(tok, &end, 10) : 0;
            if (!ok || errno == ERANGE || v < INT32_MIN || v > INT32_MAX) {
                *bad_offset = t0;
                return -1;
            }
            if (field == 0)
                rec.u = (int32_t)v;
            else
                rec.v = (int32_t)v;
        } else {
            /* %f: decimal, inf/infinity or nan; no hexadecimal forms or nan(...) payloads */
            const char *q = tok + ((tok[0] == '+' || tok[0] == '-') ? 1 : 0);
            const int hex = q[0] == '0' && (q[1] == 'x' || q[1] == 'X');
            const int paren = strchr(tok, '(') != NULL;
            float f = hex || paren ? 0.f : strtof(tok, &end);
            if (hex || paren || end != tok + tl) {
                *bad_offset = t0;
                return -1;
            }
            rec.r = f;
            if (out && ntok / 3 < cap) out[ntok / 3] = rec;
        }
        ++ntok;
    }
    if (ntok % 3 != 0) return -2;
    return ntok / 3;
}


/* ---- mf-predict criteria (test/mf.cpp:3794-4044) ------------------------------------------ */

/* mf_predict (mf.cpp:3794-3812): sequential float inner product; b out of range or NaN. */
static float or_predict(const float *P, int32_t m, const float *Q, int32_t n, int k, float b, int32_t u, int32_t v) {
    if (u < 0 || u >= m || v < 0 || v >= n) return b;
    const float *p = P + (int64_t)u * k, *q = Q + (int64_t)v * k;
    float z = 0.f;
    for (int t = 0; t < k; ++t) z = fmaf(p[t], q[t], z);
    return isnan(z) ? b : z;
}

typedef struct { int32_t row, col; float r; } or_rc;
static int or_cmp_rc(const void *a, const void *b) {
    const or_rc *x = (const or_rc *)a, *y = (const or_rc *)b;
    if (x->row != y->row) return x->row < y->row ? -1 : 1;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    return 0;
}
typedef struct { int32_t col; float pred; } or_cp;
static int or_cmp_pred(const void *a, const void *b) {
    const float x = ((const or_cp *)a)->pred, y = ((const or_cp *)b)->pred;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* calc_mpr_auc (mf.cpp:3913-4034). */
static void or_mpr_auc(const or_node *R, int64_t nnz, int32_t prob_m, int32_t prob_n, const float *P, int32_t pm,
                       const float *Q, int32_t qn, int k, float b, int transpose, double *mpr, double *auc) {
    const int32_t m = transpose ? (prob_n > qn ? prob_n : qn) : (prob_m > pm ? prob_m : pm);
    const int32_t n = transpose ? (prob_m > pm ? prob_m : pm) : (prob_n > qn ? prob_n : qn);
    or_rc *rc = (or_rc *)malloc((size_t)(nnz ? nnz : 1) * sizeof(or_rc));
    for (int64_t i = 0; i < nnz; ++i) {
        rc[i].row = transpose ? R[i].v : R[i].u;
        rc[i].col = transpose ? R[i].u : R[i].v;
        rc[i].r = R[i].r;
    }
    qsort(rc, (size_t)nnz, sizeof(or_rc), or_cmp_rc);
    int64_t *cnt = (int64_t *)calloc((size_t)m + 1, sizeof(int64_t));
    for (int64_t i = 0; i < nnz; ++i) cnt[rc[i].row + 1]++;
    for (int32_t i = 1; i < m + 1; ++i) cnt[i] += cnt[i - 1];
    or_cp *row = (or_cp *)malloc((size_t)(n ? n : 1) * sizeof(or_cp));
    int32_t *index = (int32_t *)malloc((size_t)(nnz ? nnz : 1) * sizeof(int32_t));
    int64_t total_m = 0, total_pos = 0;
    double all_mpr = 0, all_auc = 0;
    for (int32_t i = 0; i < m; ++i) {
        if (cnt[i + 1] - cnt[i] < 1) continue;
        for (int32_t j = 0; j < n; ++j) {
            row[j].col = j;
            row[j].pred = transpose ? or_predict(P, pm, Q, qn, k, b, j, i) : or_predict(P, pm, Q, qn, k, b, i, j);
        }
        int32_t pos = 0;
        for (int64_t j = cnt[i]; j < cnt[i + 1]; ++j) {
            if (rc[j].r <= 0) continue;
            index[pos++] = rc[j].col;
        }
        if (n - pos < 1 || pos < 1) continue;
        total_m++;
        total_pos += pos;
        for (int32_t q = 0; q < pos; ++q) { /* swap(row[count], row[index[k]]) (mf.cpp:3995-3999) */
            const or_cp t = row[q];
            row[q] = row[index[q]];
            row[index[q]] = t;
        }
        qsort(row, (size_t)pos, sizeof(or_cp), or_cmp_pred);
        double u_mpr = 0, u_auc = 0;
        for (int32_t g = pos; g < n; ++g) {
            if (row[pos - 1].pred <= row[g].pred) {
                u_mpr += pos;
                continue;
            }
            int32_t left = 0, right = pos - 1;
            while (left < right) {
                const int32_t mid = (left + right) / 2;
                if (row[mid].pred > row[g].pred)
                    right = mid;
                else
                    left = mid + 1;
            }
            u_mpr += left;
            u_auc += pos - left;
        }
        all_mpr += u_mpr / (n - pos);
        all_auc += u_auc / (n - pos) / pos;
    }
    *mpr = all_mpr / (double)total_pos;
    *auc = all_auc / (double)total_m;
    free(rc);
    free(cnt);
    free(row);
    free(index);
}

double or_evaluate(const or_node *R, int64_t nnz, int32_t prob_m, int32_t prob_n, const float *P, int32_t m,
                   const float *Q, int32_t n, int k, float b, int criterion) {
    if (criterion >= 10 && criterion <= 13) {
        double mpr = 0, auc = 0;
        or_mpr_auc(R, nnz, prob_m, prob_n, P, m, Q, n, k, b, criterion == 11 || criterion == 13, &mpr, &auc);
        return criterion <= 11 ? mpr : auc;
    }
    if (criterion != 0 && criterion != 1 && criterion != 2 && criterion != 5 && criterion != 6) return NAN;
    if (nnz == 0) return 0;
    double acc = 0;
    for (int64_t i = 0; i < nnz; ++i) {
        const float r = R[i].r, z = or_predict(P, m, Q, n, k, b, R[i].u, R[i].v);
        switch (criterion) {
            case 0: { const float e = r - z; acc += (double)(e * e); break; }
            case 1: acc += (double)fabsf(r - z); break;
            case 2: acc += (double)(r * logf(r / z) - r + z); break;
            case 5: acc += r > 0 ? log(1.0 + (double)expf(-z)) : log(1.0 + (double)expf(z)); break;
            default: acc += r > 0 ? (z > 0 ? 1 : 0) : (z < 0 ? 1 : 0); break;
        }
    }
    return criterion == 0 ? sqrt(acc / (double)nnz) : acc / (double)nnz;
}


/* ---- deterministic stratified schedule --------------------------------------------------- */

int64_t or_strata_epochs(const or_node *R, int64_t nnz, float *P, int32_t m, float *Q, int32_t n, int k, int kind,
                         int sr, int lanes, int G, const float *lr, int first_epoch, int n_epochs, float lambda_p,
                         float lambda_q, uint64_t seed) {
    const int64_t blocks = (int64_t)G * G;
    int64_t *off = (int64_t *)calloc((size_t)blocks + 1, sizeof(int64_t));
    or_node *S = (or_node *)malloc((size_t)(nnz ? nnz : 1) * sizeof(or_node));
    for (int64_t i = 0; i < nnz; ++i) off[((uint32_t)R[i].u % (uint32_t)G) * (uint32_t)G + (uint32_t)R[i].v % (uint32_t)G + 1]++;
    for (int64_t b = 0; b < blocks; ++b) off[b + 1] += off[b];
    int64_t *fill = (int64_t *)malloc((size_t)blocks * sizeof(int64_t));
    memcpy(fill, off, (size_t)blocks * sizeof(int64_t));
    for (int64_t i = 0; i < nnz; ++i)  /* stable counting sort */
        S[fill[((uint32_t)R[i].u % (uint32_t)G) * (uint32_t)G + (uint32_t)R[i].v % (uint32_t)G]++] = R[i];
    int64_t skipped = 0;
    int *order = (int *)malloc((size_t)G * sizeof(int));
    for (int ep = first_epoch; ep < first_epoch + n_epochs; ++ep) {
        const uint32_t round_key = (uint32_t)(or_splitmix64(seed ^ (0x5352ull << 48)) + (uint64_t)ep);
        /* strata in a seeded random order: Fisher-Yates with splitmix64 draws */
        for (int i = 0; i < G; ++i) order[i] = i;
        uint64_t h = or_splitmix64(seed ^ (0x5354ull << 48)) + (uint64_t)ep * 0x9E3779B97F4A7C15ull;
        for (int i = G - 1; i > 0; --i) {
            h = or_splitmix64(h);
            const int j = (int)(h % (uint64_t)(i + 1));
            const int t = order[i];
            order[i] = order[j];
            order[j] = t;
        }
        for (int oi = 0; oi < G; ++oi) {
            const int st = order[oi];
            for (int a = 0; a < G; ++a) {
                const int64_t blk = (int64_t)a * G + (a + st) % G;
                for (int64_t i = off[blk]; i < off[blk + 1]; ++i) {
                    const or_node x = S[i];
                    if ((uint32_t)x.u >= (uint32_t)m || (uint32_t)x.v >= (uint32_t)n) {
                        ++skipped;
                        continue;
                    }
                    const uint32_t key = sr ? (round_key ^ or_lowbias32((uint32_t)i)) : 0u;
                    update_rows(P + (int64_t)x.u * k, Q + (int64_t)x.v * k, k, x.r, lr[ep], lambda_p, lambda_q, kind,
                                sr, key, lanes, OR_DOT_LANES, 0);
                }
            }
        }
    }
    free(order);
    free(off);
    free(fill);
    free(S);
    return skipped;
}
