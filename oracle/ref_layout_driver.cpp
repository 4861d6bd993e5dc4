// ref_layout_driver.cpp - runs the reference's own host functions (compiled from
// singleGPU/sgd.cu, unmodified) on a rating file and dumps what they produce, to pin the
// oracle and the library's layout code:
//   gen_random_map x2, shuffle_problem, grid_problem, collect_data, scale_problem,
//   scale_model and shuffle_model (sgd.cu:39-134, 411-487, 593-635), plus the rand()
//   stream that the mode B / C block shuffles draw from afterwards (sgd_kernel.cu:263-267).
// time() is wrapped (-Wl,--wrap=time) so srand(time(NULL)) (sgd.cu:42) gets a fixed seed.
// TEST INFRASTRUCTURE: built by oracle/ref_build.sh into oracle/_ref/ from the reference
// sources where they lie; never part of the product.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#include <string>

#include "sgd.h"

int *gen_random_map(SGDIndex size);
void shuffle_problem(mf_problem *prob, SGDIndex *p_map, SGDIndex *q_map);
void grid_problem(mf_problem *prob);
void collect_data(mf_problem *prob, SGDRate &ave, SGDRate &std_dev);
void scale_problem(mf_problem *prob, float scale, long long u_seg, long long v_seg);
void scale_model(mf_model *model, float scale);
void shuffle_model(mf_model *model, int *inv_p_map, int *inv_q_map);

// sgd.cu calls this from sgd_train, which the driver never runs.
void sgd_update_k128(Parameter, mf_model *, mf_problem *, float) {}

static time_t g_seed = 0;
extern "C" time_t __wrap_time(time_t *t) {
    if (t) *t = g_seed;
    return g_seed;
}

static void dump(FILE *f, const void *p, size_t bytes) { fwrite(p, 1, bytes, f); }

int main(int argc, char **argv) {
    if (argc != 7) {
        fprintf(stderr, "usage: %s ratings.bin seed ux vy k out.bin\n", argv[0]);
        return 1;
    }
    g_seed = (time_t)strtoll(argv[2], nullptr, 10);
    const int ux = atoi(argv[3]), vy = atoi(argv[4]), k = atoi(argv[5]);
    FILE *in = fopen(argv[1], "rb");
    if (!in) return 2;
    fseek(in, 0, SEEK_END);
    long long nnz = ftell(in) / 12;
    rewind(in);
    mf_problem prob;
    memset(&prob, 0, sizeof(prob));
    prob.R = (mf_node *)malloc(sizeof(mf_node) * (nnz ? nnz : 1));
    if (fread(prob.R, 12, nnz, in) != (size_t)nnz) return 3;
    fclose(in);
    prob.nnz = nnz;
    prob.m = 1;
    prob.n = 1;
    for (long long i = 0; i < nnz; i++) {
        if (prob.R[i].u + 1 > prob.m) prob.m = prob.R[i].u + 1;
        if (prob.R[i].v + 1 > prob.n) prob.n = prob.R[i].v + 1;
    }
    prob.u_grid = ux; prob.v_grid = vy; prob.x_grid = 1; prob.y_grid = 1;
    prob.ux = ux; prob.vy = vy;

    float ave, std_dev;
    collect_data(&prob, ave, std_dev);
    const float scale = std::max((SGDRate)1e-4, std_dev);
    int *p_map = gen_random_map(prob.m);
    int *q_map = gen_random_map(prob.n);
    // rand() stream continuation: the first draws of the block shuffles that follow.
    std::vector<int> cont(8);
    for (int i = 0; i < 8; i++) cont[i] = i;
    std::random_shuffle(cont.begin(), cont.end());
    // (the q map was drawn after a fresh srand; re-derive nothing else here)
    shuffle_problem(&prob, p_map, q_map);
    std::vector<mf_node> shuffled(prob.R, prob.R + nnz);
    grid_problem(&prob);
    std::vector<mf_node> gridded(prob.R, prob.R + nnz);
    scale_problem(&prob, 1.0 / scale, prob.u_seg, prob.v_seg);

    // scale_model + shuffle_model on a model whose entries encode (row, col).
    mf_model model;
    memset(&model, 0, sizeof(model));
    model.m = prob.m; model.n = prob.n; model.k = k;
    model.floatp = (float *)malloc(sizeof(float) * (size_t)prob.m * k);
    model.floatq = (float *)malloc(sizeof(float) * (size_t)prob.n * k);
    for (long long i = 0; i < (long long)prob.m * k; i++) model.floatp[i] = (float)(i % 9973) * 0.001f + 0.5f;
    for (long long i = 0; i < (long long)prob.n * k; i++) model.floatq[i] = (float)(i % 7919) * 0.002f - 0.25f;
    int *inv_p = new int[prob.m], *inv_q = new int[prob.n];
    for (int i = 0; i < prob.m; i++) inv_p[p_map[i]] = i;
    for (int i = 0; i < prob.n; i++) inv_q[q_map[i]] = i;
    scale_model(&model, scale);
    shuffle_model(&model, inv_p, inv_q);

    FILE *out = fopen(argv[6], "wb");
    if (!out) return 4;
    const int32_t head[4] = {prob.m, prob.n, ux, vy};
    dump(out, head, sizeof(head));
    dump(out, &nnz, 8);
    dump(out, &ave, 4);
    dump(out, &std_dev, 4);
    dump(out, &prob.u_seg, 8);
    dump(out, &prob.v_seg, 8);
    dump(out, p_map, sizeof(int) * prob.m);
    dump(out, q_map, sizeof(int) * prob.n);
    dump(out, cont.data(), sizeof(int) * 8);
    dump(out, prob.gridSize, sizeof(long long) * ux * vy);
    dump(out, shuffled.data(), 12 * nnz);
    dump(out, gridded.data(), 12 * nnz);
    dump(out, prob.R, 12 * nnz);
    dump(out, model.floatp, sizeof(float) * (size_t)prob.m * k);
    dump(out, model.floatq, sizeof(float) * (size_t)prob.n * k);
    fclose(out);
    return 0;
}
