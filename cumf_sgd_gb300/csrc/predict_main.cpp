// predict_main.cpp - `cumf_predict -e 0 test_file model_file`, the RMSE path of LIBMF's
// mf-predict (test/mf-predict.cpp:40-133) evaluated on the GPU.  Only -e 0 (RMSE) is
// supported; the output line is the reference's "RMSE = x.xxxx".
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cumf_sgd.h"

int main(int argc, char **argv) {
    int eval = 0, i = 1;
    for (; i < argc; ++i) {
        if (strcmp(argv[i], "-e") == 0) {
            if (i + 1 >= argc) {
                printf("need to specify evaluation criterion after -e\n");
                return 1;
            }
            eval = atoi(argv[++i]);
        } else {
            break;
        }
    }
    if (eval != 0) {
        printf("only -e 0 (RMSE) is supported\n");
        return 1;
    }
    if (i >= argc - 1) {
        printf("testing data and model file not specified\n");
        return 1;
    }
    cumf_problem te;
    cumf_model model;
    if (cumf_read_problem(argv[i], 1, &te) != CUMF_OK) {
        printf("%s\n", cumf_last_error());
        return 1;
    }
    if (cumf_load_model(argv[i + 1], &model) != CUMF_OK) {
        printf("cannot load model from %s: %s\n", argv[i + 1], cumf_last_error());
        cumf_free_problem(&te);
        return 1;
    }
    double rmse = 0;
    int rc = cumf_rmse(&te, &model, &rmse);
    if (rc == CUMF_OK) printf("RMSE = %.4f\n", rmse);
    else printf("%s\n", cumf_last_error());
    cumf_free_model(&model);
    cumf_free_problem(&te);
    return rc == CUMF_OK ? 0 : 1;
}
