// predict_main.cpp - `cumf_predict [-e eval] test_file model_file [output_file]`: LIBMF's
// mf-predict (test/mf-predict.cpp:15-220) with every criterion evaluated on the GPU.  Output
// lines, messages and exit codes follow the reference: "calculating rmse ..." and
// "RMSE = x.xxxx" (and MAE, GKL,
// LOGLOSS, ACCURACY, Row-wise / Colmn-wise AUC, Row-wise / Column-wise MPR), then
// "time elapsed:...s"; argument errors print the reference's message and exit 1.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "cumf_sgd.h"

static const char *kHelp =
    "usage: mf-predict [options] test_file model_file [output_file]\n"
    "\n"
    "options:\n"
    "-e <eval>: specify the evaluation criterion (default 0)\n"
    "\t 0 -- root mean square error\n"
    "\t 1 -- mean absolute error\n"
    "\t 2 -- generalized KL-divergence\n"
    "\t 5 -- logarithmic error\n"
    "\t 6 -- accuracy\n"
    "\t10 -- row-wise mean percentile rank\n"
    "\t11 -- column-wise mean percentile rank\n"
    "\t12 -- row-wise area under the curve\n"
    "\t13 -- column-wise area under the curve\n";

static const char *label(int eval) {
    switch (eval) {
        case CUMF_EVAL_RMSE: return "RMSE = ";
        case CUMF_EVAL_MAE: return "MAE = ";
        case CUMF_EVAL_GKL: return "GKL = ";
        case CUMF_EVAL_LOGLOSS: return "LOGLOSS = ";
        case CUMF_EVAL_ACC: return "ACCURACY = ";
        case CUMF_EVAL_ROW_AUC: return "Row-wise AUC = ";
        case CUMF_EVAL_COL_AUC: return "Colmn-wise AUC = ";  // spelled as mf-predict.cpp:167
        case CUMF_EVAL_ROW_MPR: return "Row-wise MPR = ";
        case CUMF_EVAL_COL_MPR: return "Column-wise MPR = ";
        default: return NULL;
    }
}

int main(int argc, char **argv) {
    if (argc == 1) {
        printf("%s\n", kHelp);
        return 1;
    }
    int eval = CUMF_EVAL_RMSE, i = 1;
    for (; i < argc; ++i) {
        if (strcmp(argv[i], "-e") == 0) {
            if (i + 1 >= argc) {
                printf("need to specify evaluation criterion after -e\n");
                return 1;
            }
            eval = atoi(argv[++i]);
            if (!label(eval)) {
                printf("unknown evaluation criterion\n");
                return 1;
            }
        } else {
            break;
        }
    }
    if (i >= argc - 1) {
        printf("testing data and model file not specified\n");
        return 1;
    }
    if (argc - i > 3) {  // test, model and at most one output path (mf-predict.cpp:78-95)
        printf("invalid argument\n");
        return 1;
    }
    cumf_problem te;
    cumf_model model;
    if (cumf_read_problem(argv[i], 1, &te) != CUMF_OK) {
        printf("%s\n", cumf_last_error());
        return 1;
    }
    if (cumf_load_model(argv[i + 1], &model) != CUMF_OK) {
        printf("cannot load model from %s\n", argv[i + 1]);
        cumf_free_problem(&te);
        return 1;
    }
    const clock_t start = clock();
    if (eval == CUMF_EVAL_RMSE) printf("calculating rmse ...\n");  // calc_rmse's line (mf.cpp:3817)
    double v = 0;
    int rc = cumf_evaluate(&te, &model, eval, &v);
    if (rc == CUMF_OK) {
        printf("%s%.4f\n", label(eval), v);
        printf("time elapsed:%.8lfs\n", (clock() - start) / (double)CLOCKS_PER_SEC);
    } else {
        printf("%s\n", cumf_last_error());
    }
    cumf_free_model(&model);
    cumf_free_problem(&te);
    return rc == CUMF_OK ? 0 : 1;
}
