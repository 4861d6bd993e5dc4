// api_io.cpp - host side of the C ABI: errors, parameters, the CLI parser, rating and
// model files, the id shuffle and the u x v grid partitioner.
#include <cuda_runtime.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <memory>
#include <cctype>
#include <cmath>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "cumf_sgd.h"
#include "glibc_shuffle.h"
#include "internal.h"

namespace cumf {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
    set_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    int code = CUMF_ERR_CUDA;
    if (e == cudaErrorMemoryAllocation) code = CUMF_ERR_NOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) code = CUMF_ERR_NODEVICE;
    return fail(code, msg);
}

// Host buffers: page-locked when asked and possible, else plain malloc.
//
// Page-locked blocks are cached: a pinned buffer given back by cumf_free_model or
// cumf_free_problem is kept, and the next pinned request it fits (between half its size and
// its size) takes it again.  Page-locking costs about 30 ms per GB on the GB300 host (8 ms
// for a 480,189 x 17,770 x 128 model), which repeated training calls then pay once.  At most
// 2 GB stay cached (the environment variable CUMF_HOST_CACHE_MB sets another limit, 0 turns
// the cache off); cumf_release_host_cache gives them back to the system.
namespace {
size_t pinned_cache_limit() {
    static const size_t limit = [] {
        const char *e = getenv("CUMF_HOST_CACHE_MB");
        if (!e || !*e) return size_t(2) << 30;
        const long long mb = atoll(e);
        return mb > 0 ? (size_t)mb << 20 : size_t(0);
    }();
    return limit;
}
struct PinnedCache {
    std::mutex mu;
    std::vector<std::pair<void *, size_t>> free_blocks;  // cached, not in use
    std::vector<std::pair<void *, size_t>> live;         // handed out
    size_t cached_bytes = 0;
};
PinnedCache &pinned_cache() {
    static PinnedCache *c = new PinnedCache();  // never destroyed: blocks may be freed at exit
    return *c;
}
}  // namespace

static void *host_alloc(size_t bytes, int *pinned) {
    if (bytes == 0) bytes = 1;
    if (*pinned) {
        PinnedCache &c = pinned_cache();
        {
            std::lock_guard<std::mutex> lock(c.mu);
            size_t best = SIZE_MAX;
            int at = -1;
            for (size_t i = 0; i < c.free_blocks.size(); ++i) {
                const size_t cap = c.free_blocks[i].second;
                if (cap >= bytes && cap / 2 <= bytes && cap < best) {
                    best = cap;
                    at = (int)i;
                }
            }
            if (at >= 0) {
                auto blk = c.free_blocks[at];
                c.free_blocks.erase(c.free_blocks.begin() + at);
                c.cached_bytes -= blk.second;
                c.live.push_back(blk);
                return blk.first;
            }
        }
        void *p = nullptr;
        if (cudaMallocHost(&p, bytes) == cudaSuccess) {
            std::lock_guard<std::mutex> lock(c.mu);
            c.live.push_back({p, bytes});
            return p;
        }
        cudaGetLastError();  // clear; fall back to pageable memory
        *pinned = 0;
    }
    return malloc(bytes);
}

static void host_free(void *p, int pinned) {
    if (!p) return;
    if (!pinned) {
        free(p);
        return;
    }
    PinnedCache &c = pinned_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    for (size_t i = 0; i < c.live.size(); ++i) {
        if (c.live[i].first != p) continue;
        const auto blk = c.live[i];
        c.live.erase(c.live.begin() + i);
        if (c.cached_bytes + blk.second <= pinned_cache_limit()) {
            c.free_blocks.push_back(blk);
            c.cached_bytes += blk.second;
            return;
        }
        break;
    }
    cudaFreeHost(p);
}

extern "C" int cumf_release_host_cache(void) {
    PinnedCache &c = pinned_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    for (auto &blk : c.free_blocks) cudaFreeHost(blk.first);
    c.free_blocks.clear();
    c.cached_bytes = 0;
    return CUMF_OK;
}

// Block g's walk (sgd.cu:466-481): its slots from the first one not yet filled by earlier
// blocks' swaps; the record held at the walk position either belongs to g (it stays, the walk
// advances) or goes to the next free slot of its own block, whose original record is taken
// in its place.  Slots at or past a block's free pointer still hold their original records,
// so only the original block ids are read.
void grid_order(const int32_t *bid, int64_t nnz, int G, const int64_t *grid_size, int64_t *fin) {
    std::vector<int64_t> begin(G + 1, 0), free_slot(G);
    for (int g = 0; g < G; ++g) begin[g + 1] = begin[g] + grid_size[g];
    for (int g = 0; g < G; ++g) free_slot[g] = begin[g];
    if (nnz <= 0) return;
    for (int g = 0; g < G; ++g) {
        int64_t p = free_slot[g];
        const int64_t end = begin[g + 1];
        if (p >= end) continue;
        int64_t cur = p;  // original index of the record held at the walk position
        while (true) {
            const int c = bid[cur];
            if (c == g) {
                fin[p] = cur;
                if (++p >= end) break;
                cur = p;
            } else {
                const int64_t slot = free_slot[c]++;
                fin[slot] = cur;
                cur = slot;
            }
        }
    }
}

}  // namespace cumf

using namespace cumf;

extern "C" {

int cumf_abi_version(void) { return CUMF_ABI_VERSION; }

const char *cumf_last_error(void) { return g_last_error.c_str(); }

int cumf_default_params(cumf_params *p) {
    if (!p) return fail(CUMF_ERR_ARG, "params is NULL");
    memset(p, 0, sizeof(*p));
    // Parameter() defaults, singleGPU/sgd.h:45.
    p->k = 80;
    p->num_workers = 12;
    p->u_grid = p->v_grid = p->x_grid = p->y_grid = 1;
    p->ux = p->vy = 1;
    p->num_iters = 30;
    p->gpu = 3;
    p->lambda_p = 0.05f;
    p->lambda_q = 0.05f;
    p->lrate = 0.0f;
    p->alpha = 0.01f;
    p->beta = 0.01f;
    p->seed = 0;
    p->precision = CUMF_FP16;
    p->lanes = 0;
    p->quiet = 0;
    p->epochs_per_launch = 0;
    p->verbose_epochs = 0;
    p->prefetch = -1;
    p->l2_hints = -1;
    p->ring = -1;
    p->hot_rows = kHotDefaultConcurrency;
    return CUMF_OK;
}

// is_numerical (singleGPU/main.cpp:21-31): true when the string holds at least one digit.
static bool is_numerical(const char *s) {
    if (!s) return false;
    int c = 0;
    for (; *s; ++s)
        if (isdigit((unsigned char)*s)) ++c;
    return c > 0;
}

static int copy_path(char *dst, const std::string &src) {
    if (src.size() >= 1024) return fail(CUMF_ERR_ARG, "path too long: " + src);
    memcpy(dst, src.c_str(), src.size() + 1);
    return CUMF_OK;
}

int cumf_parse_args(int argc, char **argv, cumf_args *out) {
    if (!out) return fail(CUMF_ERR_ARG, "args is NULL");
    memset(out, 0, sizeof(*out));
    cumf_default_params(&out->param);
    cumf_params &p = out->param;
    if (argc <= 1 || !argv) return fail(CUMF_ERR_ARG, "error");
    std::vector<std::string> args(argv, argv + argc);
    auto need = [&](int i, const char *msg) -> bool { return (i + 1) < argc || (fail(CUMF_ERR_ARG, msg), false); };
    int i;
    for (i = 1; i < argc; ++i) {
        const std::string &a = args[i];
        if (a == "-g") {
            if (!need(i, "need to specify the id of GPUs after -g")) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i])) return fail(CUMF_ERR_ARG, "-g should be followed by a number");
            p.gpu = atoi(argv[i]);
        } else if (a == "-l") {
            if (!need(i, "need to specify lambda after -l")) return CUMF_ERR_ARG;
            ++i;
            // "-l p[,q]" (main.cpp:57-77); strtok semantics on a private copy.
            std::string v = args[i];
            size_t comma = v.find(',');
            std::string first = v.substr(0, comma);
            if (!is_numerical(first.c_str()))
                return fail(CUMF_ERR_ARG, "regularization coefficient should be a number");
            p.lambda_p = p.lambda_q = (float)strtod(first.c_str(), nullptr);
            if (comma != std::string::npos) {
                std::string second = v.substr(comma + 1);
                size_t c2 = second.find(',');
                if (c2 != std::string::npos) second = second.substr(0, c2);
                if (!second.empty()) {
                    if (!is_numerical(second.c_str()))
                        return fail(CUMF_ERR_ARG, "regularization coefficient should be a number");
                    p.lambda_q = (float)strtod(second.c_str(), nullptr);
                }
            }
        } else if (a == "-k") {
            if (!need(i, "need to specify number of factors after -k")) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i])) return fail(CUMF_ERR_ARG, "-k should be followed by a number");
            p.k = atoi(argv[i]);
        } else if (a == "-t") {
            if (!need(i, "need to specify number of iterations after -t")) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i])) return fail(CUMF_ERR_ARG, "-i should be followed by a number");
            p.num_iters = atoi(argv[i]);
        } else if (a == "-r") {
            if (!need(i, "need to specify eta after -r")) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i])) return fail(CUMF_ERR_ARG, "-r should be followed by a number");
            p.lrate = (float)atof(argv[i]);
        } else if (a == "-a") {
            if (!need(i, "need to specify eta after -a")) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i])) return fail(CUMF_ERR_ARG, "-a should be followed by a number");
            p.alpha = (float)atof(argv[i]);
        } else if (a == "-b") {
            if (!need(i, "need to specify eta after -b")) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i])) return fail(CUMF_ERR_ARG, "-b should be followed by a number");
            p.beta = (float)atof(argv[i]);
        } else if (a == "-s") {
            if (!need(i, "need to specify number of parallel workers after -s(multiples of 4)")) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i]))
                return fail(CUMF_ERR_ARG, "-s should be followed by a number which is multiple of 4");
            p.num_workers = ((atoi(argv[i]) + 3) / 4) * 4;  // main.cpp:139
        } else if (a == "-u" || a == "-v" || a == "-x" || a == "-y") {
            const char c = a[1];
            std::string msg = std::string("need to specify number of ") + c + " grid after -" + c;
            if (!need(i, msg.c_str())) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i]))
                return fail(CUMF_ERR_ARG, std::string("-") + c + " should be followed by a number");
            const int val = atoi(argv[i]);
            if (c == 'u') p.u_grid = val;
            if (c == 'v') p.v_grid = val;
            if (c == 'x') p.x_grid = val;
            if (c == 'y') p.y_grid = val;
        } else if (a == "-p") {
            if (i == argc - 1) return fail(CUMF_ERR_ARG, "need to specify path after -p");
            ++i;
            if (int rc = copy_path(out->va_path, args[i])) return rc;
        } else if (a == "--seed") {
            if (!need(i, "need to specify a number after --seed")) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i])) return fail(CUMF_ERR_ARG, "--seed should be followed by a number");
            p.seed = strtoull(argv[i], nullptr, 10);
        } else if (a == "--precision") {
            if (!need(i, "need to specify fp16|bf16|fp32|bf16sr|fp16sr after --precision")) return CUMF_ERR_ARG;
            ++i;
            const std::string v = args[i];
            if (v == "fp16") p.precision = CUMF_FP16;
            else if (v == "bf16") p.precision = CUMF_BF16;
            else if (v == "fp32") p.precision = CUMF_FP32;
            else if (v == "bf16sr") p.precision = CUMF_BF16_SR;
            else if (v == "fp16sr") p.precision = CUMF_FP16_SR;
            else return fail(CUMF_ERR_ARG, "unknown precision " + v);
        } else if (a == "--lanes") {
            if (!need(i, "need to specify a number after --lanes")) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i])) return fail(CUMF_ERR_ARG, "--lanes should be followed by a number");
            p.lanes = atoi(argv[i]);
        } else if (a == "--quiet") {
            p.quiet = 1;
        } else if (a == "--deterministic") {
            if (!need(i, "need to specify a number after --deterministic")) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i])) return fail(CUMF_ERR_ARG, "--deterministic should be followed by a number");
            p.deterministic = atoi(argv[i]);
        } else if (a == "--hot-rows") {
            if (!need(i, "need to specify a number after --hot-rows")) return CUMF_ERR_ARG;
            ++i;
            if (!is_numerical(argv[i])) return fail(CUMF_ERR_ARG, "--hot-rows should be followed by a number");
            p.hot_rows = (float)atof(argv[i]);
            if (!(p.hot_rows >= 0.f)) return fail(CUMF_ERR_ARG, "--hot-rows should be 0 or more");
        } else {
            break;
        }
    }
    if (i >= argc) return fail(CUMF_ERR_ARG, "training data not specified");
    if (int rc = copy_path(out->tr_path, args[i++])) return rc;
    std::string model_path;
    if (i < argc) {
        model_path = args[i];
    } else {
        // basename(train) + ".model" (main.cpp:205-213)
        const std::string &tr = args[i - 1];
        size_t slash = tr.rfind('/');
        model_path = (slash == std::string::npos ? tr : tr.substr(slash + 1)) + ".model";
    }
    if (int rc = copy_path(out->model_path, model_path)) return rc;
    if (p.u_grid * p.v_grid == 1) {  // main.cpp:219-223
        p.x_grid = 1;
        p.y_grid = 1;
    }
    p.ux = p.u_grid * p.x_grid;
    p.vy = p.v_grid * p.y_grid;
    return CUMF_OK;
}

// ---- rating files ------------------------------------------------------------------

int cumf_alloc_problem(int64_t nnz, int pinned, cumf_problem *out) {
    if (!out || nnz < 0) return fail(CUMF_ERR_ARG, "bad problem allocation request");
    memset(out, 0, sizeof(*out));
    int pin = pinned ? 1 : 0;
    out->R = (cumf_node *)host_alloc((size_t)nnz * sizeof(cumf_node), &pin);
    if (!out->R) return fail(CUMF_ERR_NOMEM, "cannot allocate rating buffer");
    out->pinned = pin;
    out->nnz = nnz;
    out->m = 1;
    out->n = 1;
    return CUMF_OK;
}

int cumf_free_problem(cumf_problem *prob) {
    if (!prob) return CUMF_OK;
    host_free(prob->R, prob->pinned);
    prob->R = nullptr;
    prob->nnz = 0;
    return CUMF_OK;
}

// Reads whole 12-byte records of one file into R (records [0, count)); returns the
// number read, or -1 on an I/O error.
static int64_t read_records(const std::string &path, cumf_node *R, int64_t count) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return -1;
    int64_t done = 0;
    while (done < count) {
        size_t got = fread(R + done, sizeof(cumf_node), (size_t)std::min<int64_t>(count - done, 1 << 20), f);
        if (got == 0) break;
        done += (int64_t)got;
    }
    fclose(f);
    return done;
}

static int64_t file_size(const std::string &path) {
    struct stat st;
    if (stat(path.c_str(), &st) != 0) return -1;
    return (int64_t)st.st_size;
}

// m, n from the records in parallel; negative ids are an error.
static int scan_extent(const cumf_node *R, int64_t nnz, int32_t *m, int32_t *n) {
    const int T = (int)std::max<unsigned>(1u, std::min<unsigned>(16u, std::thread::hardware_concurrency()));
    std::vector<int32_t> mm(T, 1), nn(T, 1);
    std::vector<int64_t> neg(T, -1);
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t) {
        th.emplace_back([&, t] {
            const int64_t a = nnz * t / T, b = nnz * (t + 1) / T;
            int32_t lm = 1, ln = 1;
            for (int64_t i = a; i < b; ++i) {
                const int32_t u = R[i].u, v = R[i].v;
                if (u < 0 || v < 0) {
                    if (neg[t] < 0) neg[t] = i;
                    continue;
                }
                if (u + 1 > lm) lm = u + 1;
                if (v + 1 > ln) ln = v + 1;
            }
            mm[t] = lm;
            nn[t] = ln;
        });
    }
    for (auto &x : th) x.join();
    int32_t M = 1, N = 1;
    for (int t = 0; t < T; ++t) {
        if (neg[t] >= 0)
            return fail(CUMF_ERR_FORMAT, "negative user or item id in record " + std::to_string(neg[t]));
        M = std::max(M, mm[t]);
        N = std::max(N, nn[t]);
    }
    *m = M;
    *n = N;
    return CUMF_OK;
}

int cumf_read_problem(const char *path, int pinned, cumf_problem *out) {
    if (!out) return fail(CUMF_ERR_ARG, "problem is NULL");
    memset(out, 0, sizeof(*out));
    out->m = out->n = 1;
    if (!path || !*path) return fail(CUMF_ERR_IO, "file  open failed");
    const std::string base(path);
    // Shards path0 .. path79 (sgd.cu:207-217).
    std::vector<std::string> shards;
    for (int i = 0; i < 80; ++i) {
        std::string s = base + std::to_string(i);
        if (access(s.c_str(), F_OK) != -1) shards.push_back(s);
    }
    std::vector<std::string> files = shards.empty() ? std::vector<std::string>{base} : shards;
    std::vector<int64_t> counts(files.size()), offsets(files.size() + 1, 0);
    for (size_t i = 0; i < files.size(); ++i) {
        const int64_t sz = file_size(files[i]);
        if (sz < 0) return fail(CUMF_ERR_IO, "file " + files[i] + " open failed");
        counts[i] = sz / 12;  // trailing partial record ignored (sgd.cu:237)
        offsets[i + 1] = offsets[i] + counts[i];  // offset_list[0] = 0 (uninitialised in sgd.cu:293-296)
    }
    const int64_t nnz = offsets[files.size()];
    if (int rc = cumf_alloc_problem(nnz, pinned, out)) return rc;
    std::vector<int64_t> got(files.size(), 0);
    std::vector<std::thread> th;
    for (size_t i = 0; i < files.size(); ++i)
        th.emplace_back([&, i] { got[i] = read_records(files[i], out->R + offsets[i], counts[i]); });
    for (auto &x : th) x.join();
    for (size_t i = 0; i < files.size(); ++i) {
        if (got[i] != counts[i]) {
            cumf_free_problem(out);
            return fail(CUMF_ERR_IO, "short read from " + files[i]);
        }
    }
    int rc = scan_extent(out->R, nnz, &out->m, &out->n);
    if (rc) {
        cumf_free_problem(out);
        return rc;
    }
    return CUMF_OK;
}

int cumf_write_problem(const char *path, const cumf_problem *prob) {
    if (!path || !prob || (prob->nnz > 0 && !prob->R)) return fail(CUMF_ERR_ARG, "bad write_problem arguments");
    FILE *f = fopen(path, "wb");
    if (!f) return fail(CUMF_ERR_IO, std::string("cannot open ") + path + " for writing");
    size_t w = prob->nnz ? fwrite(prob->R, sizeof(cumf_node), (size_t)prob->nnz, f) : 0;
    int c = fclose(f);
    if (w != (size_t)prob->nnz || c != 0) return fail(CUMF_ERR_IO, std::string("write failed: ") + path);
    return CUMF_OK;
}

// ---- model files -------------------------------------------------------------------

int cumf_alloc_model(int32_t m, int32_t n, int32_t k, cumf_model *out) {
    if (!out || m < 0 || n < 0 || k <= 0) return fail(CUMF_ERR_ARG, "bad model allocation request");
    memset(out, 0, sizeof(*out));
    int pin = 1;
    out->P = (float *)host_alloc((size_t)m * k * sizeof(float), &pin);
    int pin2 = pin;
    out->Q = (float *)host_alloc((size_t)n * k * sizeof(float), &pin2);
    if (pin2 != pin) {  // keep one flag for both buffers
        host_free(out->Q, pin2);
        int p0 = 0;
        out->Q = (float *)host_alloc((size_t)n * k * sizeof(float), &p0);
        if (pin) {
            host_free(out->P, pin);
            out->P = (float *)host_alloc((size_t)m * k * sizeof(float), &p0);
        }
        pin = 0;
    }
    if (!out->P || !out->Q) {
        cumf_free_model(out);
        return fail(CUMF_ERR_NOMEM, "cannot allocate model");
    }
    out->pinned = pin;
    out->fun = 0;
    out->m = m;
    out->n = n;
    out->k = k;
    return CUMF_OK;
}

int cumf_free_model(cumf_model *model) {
    if (!model) return CUMF_OK;
    host_free(model->P, model->pinned);
    host_free(model->Q, model->pinned);
    model->P = model->Q = nullptr;
    return CUMF_OK;
}

int cumf_save_model(const cumf_model *model, const char *path) {
    if (!model || !path || !*path) return fail(CUMF_ERR_ARG, "bad save_model arguments");
    FILE *f = fopen(path, "wb");  // truncates, replacing the reference's `rm -f` (main.cpp:237-239)
    if (!f) return fail(CUMF_ERR_IO, std::string("save model failed: cannot open ") + path);
    const int32_t head[4] = {0, model->m, model->n, model->k};
    bool ok = fwrite(head, sizeof(int32_t), 4, f) == 4;
    ok = ok && fwrite(&model->b, sizeof(float), 1, f) == 1;
    const size_t np = (size_t)model->m * model->k, nq = (size_t)model->n * model->k;
    ok = ok && (np == 0 || fwrite(model->P, sizeof(float), np, f) == np);
    ok = ok && (nq == 0 || fwrite(model->Q, sizeof(float), nq, f) == nq);
    ok = (fclose(f) == 0) && ok;
    if (!ok) return fail(CUMF_ERR_IO, std::string("write failed: ") + path);
    return CUMF_OK;
}

int cumf_load_model(const char *path, cumf_model *out) {
    if (!out || !path) return fail(CUMF_ERR_ARG, "bad load_model arguments");
    memset(out, 0, sizeof(*out));
    FILE *f = fopen(path, "rb");
    if (!f) return fail(CUMF_ERR_IO, std::string(path) + " open failed");
    int32_t head[4];
    float b;
    if (fread(head, sizeof(int32_t), 4, f) != 4 || fread(&b, sizeof(float), 1, f) != 1) {
        fclose(f);
        return fail(CUMF_ERR_FORMAT, std::string("truncated model header: ") + path);
    }
    const int32_t m = head[1], n = head[2], k = head[3];
    if (m < 0 || n < 0 || k <= 0) {
        fclose(f);
        return fail(CUMF_ERR_FORMAT, std::string("bad model header: ") + path);
    }
    const int64_t want = 20 + 4ll * k * ((int64_t)m + n);
    const int64_t have = file_size(path);
    if (have != want) {
        fclose(f);
        return fail(CUMF_ERR_FORMAT, std::string("model file has ") + std::to_string(have) +
                                         " bytes, header implies " + std::to_string(want));
    }
    if (int rc = cumf_alloc_model(m, n, k, out)) {
        fclose(f);
        return rc;
    }
    out->fun = head[0];
    out->b = b;
    const size_t np = (size_t)m * k, nq = (size_t)n * k;
    bool ok = (np == 0 || fread(out->P, sizeof(float), np, f) == np);
    ok = ok && (nq == 0 || fread(out->Q, sizeof(float), nq, f) == nq);
    fclose(f);
    if (!ok) {
        cumf_free_model(out);
        return fail(CUMF_ERR_IO, std::string("short read: ") + path);
    }
    return CUMF_OK;
}

// ---- shuffle and grid ----------------------------------------------------------------

int cumf_random_map(uint32_t seed, int32_t size, int32_t *map) {
    if (size < 0 || (size > 0 && !map)) return fail(CUMF_ERR_ARG, "bad random_map arguments");
    GlibcRand rng(seed);
    for (int32_t i = 0; i < size; ++i) map[i] = i;
    glibc_random_shuffle(map, size, rng);
    return CUMF_OK;
}

int cumf_grid_problem(cumf_node *R, int64_t nnz, int32_t m, int32_t n, int ux, int vy,
                      int64_t *grid_size, int64_t *u_seg_out, int64_t *v_seg_out) {
    if (ux < 1 || vy < 1 || (nnz > 0 && !R) || !grid_size)
        return fail(CUMF_ERR_ARG, "bad grid_problem arguments");
    // Segment sizes (sgd.cu:419-426).
    const int64_t u_seg = ux == 1 ? m : (int64_t)ceil((double)m / ux);
    const int64_t v_seg = vy == 1 ? n : (int64_t)ceil((double)n / vy);
    if (u_seg_out) *u_seg_out = u_seg;
    if (v_seg_out) *v_seg_out = v_seg;
    const int G = ux * vy;
    // Block ids (u / u_seg) * vy + v / v_seg in 32-bit unsigned arithmetic, and the counts.
    const uint32_t us = (uint32_t)std::max<int64_t>(1, u_seg), vs = (uint32_t)std::max<int64_t>(1, v_seg);
    std::unique_ptr<int32_t[]> bid(new int32_t[(size_t)std::max<int64_t>(1, nnz)]);  // filled by the threads
    std::vector<std::vector<int64_t>> part(16, std::vector<int64_t>(G, 0));
    std::vector<int> bad(16, 0);
    parallel_chunks(nnz, [&](int64_t a, int64_t b, int t) {
        for (int64_t i = a; i < b; ++i) {
            const cumf_node x = R[i];
            const int64_t g = (x.u < 0 || x.v < 0) ? G : (int64_t)((uint32_t)x.u / us) * vy + (int64_t)((uint32_t)x.v / vs);
            if (g >= G) {
                bad[t] = 1;
                bid[i] = 0;
                continue;
            }
            bid[i] = (int32_t)g;
            ++part[t][g];
        }
    });
    for (int t = 0; t < 16; ++t)
        if (bad[t]) return fail(CUMF_ERR_RANGE, "rating outside the grid");
    for (int g = 0; g < G; ++g) {
        grid_size[g] = 0;
        for (int t = 0; t < 16; ++t) grid_size[g] += part[t][g];
    }
    // The reference's cycle-swap order, replayed on the ids, then one gather of the records.
    std::unique_ptr<int64_t[]> fin(new int64_t[(size_t)std::max<int64_t>(1, nnz)]);
    parallel_chunks(nnz, [&](int64_t a, int64_t b, int) {  // map the pages on all threads first
        if (b > a) memset(fin.get() + a, 0, (size_t)(b - a) * sizeof(int64_t));
    });
    grid_order(bid.get(), nnz, G, grid_size, fin.get());
    std::unique_ptr<cumf_node[]> tmp(new cumf_node[(size_t)std::max<int64_t>(1, nnz)]);
    parallel_chunks(nnz, [&](int64_t a, int64_t b, int) {
        for (int64_t i = a; i < b; ++i) tmp[i] = R[fin[i]];
    });
    parallel_chunks(nnz, [&](int64_t a, int64_t b, int) {
        if (b > a) memcpy(R + a, tmp.get() + a, (size_t)(b - a) * sizeof(cumf_node));
    });
    return CUMF_OK;
}

int64_t cumf_batches_per_worker(int64_t nnz, int num_workers) {
    if (num_workers <= 0 || nnz < 0) return 0;
    return batches_per_worker(nnz, num_workers);
}

int cumf_lr_schedule(float alpha, float beta, float lrate, int n, float *out) {
    if (n < 0 || (n > 0 && !out)) return fail(CUMF_ERR_ARG, "bad lr_schedule arguments");
    for (int i = 0; i < n; ++i) {
        // sgd_kernel.cu:144-149: computed in double, stored as float.
        double r = alpha / (1 + beta * pow((double)i, 1.5)) + lrate;
        out[i] = (float)r;
    }
    return CUMF_OK;
}

}  // extern "C"
