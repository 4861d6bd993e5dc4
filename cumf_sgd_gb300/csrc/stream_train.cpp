// stream_train.cpp - modes B and C of sgd_update_k128: ratings and factors in host memory,
// u x v (and x x y) blocks streamed through the device.
#include <cuda_runtime.h>

#include "cumf_sgd.h"
#include "internal.h"

namespace cumf {

int stream_train(const cumf_problem *tr, const cumf_params &p, int workers, int lanes,
                 cumf_model *out, cumf_train_stats *st) {
    (void)tr;
    (void)p;
    (void)workers;
    (void)lanes;
    (void)out;
    (void)st;
    return fail(CUMF_ERR_ARG, "u*v > 1 is not built yet");
}

}  // namespace cumf
