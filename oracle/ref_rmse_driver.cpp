// ref_rmse_driver.cpp - prints calc_rmse (test/mf.cpp:3815-3839) with full precision for a
// test file and a model file, using the reference LIBMF sources compiled unmodified.
// TEST INFRASTRUCTURE: built by oracle/ref_build.sh into oracle/_ref/.
#include <cstdio>
#include <string>
#include "mf.h"
using namespace mf;
int main(int argc, char **argv) {
    if (argc != 3) { fprintf(stderr, "usage: %s test.bin model\n", argv[0]); return 1; }
    mf::mf_problem prob = mf::read_problem(std::string(argv[1]));
    mf_model *model = mf_load_model(argv[2]);
    if (!model) return 2;
    double r = calc_rmse(&prob, model);
    printf("RMSE_FULL %.17g\n", r);
    return 0;
}
