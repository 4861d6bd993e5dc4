// cli_main.cpp - the `cumf_sgd` command line, a drop-in for singleGPU/main.cpp:275-321.
//
//   cumf_sgd [-g id] [-l lp[,lq]] [-k 128] [-t iters] [-r lrate] [-a alpha] [-b beta]
//            [-s workers] [-u U] [-v V] [-x X] [-y Y] [-p test_file]
//            [--seed N] [--precision fp16|bf16|fp32|bf16sr|fp16sr] [--lanes N] [--quiet]
//            train_file [model_file]
//
// Exit status 1 on bad arguments (main.cpp:286-289); unlike the reference, a failed read,
// training or model write also exits non-zero with the library's message.  With -p the
// test RMSE is printed after each epoch (the reference parses -p but never reads it).
#include <stdio.h>
#include <string.h>

#include "cumf_sgd.h"

int main(int argc, char **argv) {
    cumf_args arg;
    if (cumf_parse_args(argc, argv, &arg) != CUMF_OK) {
        printf("%s\n", cumf_last_error());
        return 1;
    }
    cumf_problem tr, va;
    memset(&va, 0, sizeof(va));
    if (cumf_read_problem(arg.tr_path, 1, &tr) != CUMF_OK) {
        printf("%s\n", cumf_last_error());
        return 2;
    }
    if (!arg.param.quiet) printf("m:%d, n:%d, nnz:%lld\n", tr.m, tr.n, (long long)tr.nnz);
    const bool have_va = arg.va_path[0] != '\0';
    if (have_va) {
        if (cumf_read_problem(arg.va_path, 1, &va) != CUMF_OK) {
            printf("%s\n", cumf_last_error());
            cumf_free_problem(&tr);
            return 2;
        }
        arg.param.verbose_epochs = 1;
    }
    cumf_model model;
    cumf_train_stats st;
    int rc = cumf_train(&tr, have_va ? &va : nullptr, &arg.param, &model, &st);
    if (rc != CUMF_OK) {
        printf("training failed: %s\n", cumf_last_error());
        cumf_free_problem(&tr);
        cumf_free_problem(&va);
        return 3;
    }
    if (!arg.param.quiet) printf("save_model() is called\n");
    rc = cumf_save_model(&model, arg.model_path);
    if (rc != CUMF_OK) printf("%s\n", cumf_last_error());
    cumf_free_model(&model);
    cumf_free_problem(&tr);
    cumf_free_problem(&va);
    if (!arg.param.quiet) printf("\ntraining application finished...\n\n\n");
    return rc == CUMF_OK ? 0 : 4;
}
