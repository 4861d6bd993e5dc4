// cli_main.cpp - the `cumf_sgd` command line, a drop-in for singleGPU/main.cpp:275-321.
//
//   cumf_sgd [-g id] [-l lp[,lq]] [-k 128] [-t iters] [-r lrate] [-a alpha] [-b beta]
//            [-s workers] [-u U] [-v V] [-x X] [-y Y] [-p test_file]
//            [--seed N] [--precision fp16|bf16|fp32|bf16sr|fp16sr] [--lanes N] [--quiet]
//            [--checkpoint path [--checkpoint-every N] [--resume]] [--deterministic G]
//            [--hot-rows X] train_file [model_file]
//
// Exit status 1 on bad arguments (main.cpp:286-289); unlike the reference, a failed read,
// training or model write also exits non-zero with the library's message.  With -p the
// test RMSE is printed after each epoch (the reference parses -p but never reads it).
// --checkpoint writes the in-HBM factors every N epochs (default 1; mode A only) and
// --resume continues from a matching checkpoint (cumf_train_ckpt).  --deterministic 1 (or a
// grid size G) trains with the bit-reproducible stratified schedule instead of batch-Hogwild.
// --hot-rows X gives the most-rated rows copies for about X workers each (0.5 suits skewed
// item popularity; the default 0 keeps the reference's update, one row per rating).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "cumf_sgd.h"

int main(int argc, char **argv) {
    // Checkpoint flags are taken out before the reference flags are parsed.
    cumf_checkpoint ck;
    memset(&ck, 0, sizeof(ck));
    ck.every = 1;
    std::vector<char *> rest;
    for (int i = 0; i < argc; ++i) {
        if (strcmp(argv[i], "--checkpoint") == 0 || strcmp(argv[i], "--checkpoint-every") == 0) {
            if (i + 1 >= argc) {
                printf("error: %s needs a value\n", argv[i]);
                return 1;
            }
            if (argv[i][12] == '\0')
                ck.path = argv[++i];
            else
                ck.every = atoi(argv[++i]);
        } else if (strcmp(argv[i], "--resume") == 0) {
            ck.resume = 1;
        } else {
            rest.push_back(argv[i]);
        }
    }
    if ((ck.resume || ck.every != 1) && !ck.path) {
        printf("error: --resume and --checkpoint-every need --checkpoint\n");
        return 1;
    }
    argc = (int)rest.size();
    argv = rest.data();
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
    int rc = ck.path ? cumf_train_ckpt(&tr, have_va ? &va : nullptr, &arg.param, &ck, &model, &st, nullptr)
                     : cumf_train(&tr, have_va ? &va : nullptr, &arg.param, &model, &st);
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
