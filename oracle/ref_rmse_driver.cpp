// ref_rmse_driver.cpp - prints the evaluation criteria of test/mf.cpp (calc_rmse :3815,
// calc_mae :3841, calc_gkl :3857, calc_logloss :3874, calc_accuracy :3894, calc_mpr :4036,
// calc_auc :4041) with full precision for a test file and a model file, using the reference
// LIBMF sources compiled unmodified.  calc_mpr/calc_auc sort the problem in place, so the
// problem is read again before each of them.
// TEST INFRASTRUCTURE: built by oracle/ref_build.sh into oracle/_ref/.
#include <cstdio>
#include <string>
#include "mf.h"
using namespace mf;
int main(int argc, char **argv) {
    if (argc != 3 && argc != 4) { fprintf(stderr, "usage: %s test.bin model [all]\n", argv[0]); return 1; }
    mf::mf_problem prob = mf::read_problem(std::string(argv[1]));
    mf_model *model = mf_load_model(argv[2]);
    if (!model) return 2;
    double r = calc_rmse(&prob, model);
    printf("RMSE_FULL %.17g\n", r);
    if (argc == 4) {
        printf("CRIT 1 %.17g\n", calc_mae(&prob, model));
        printf("CRIT 2 %.17g\n", calc_gkl(&prob, model));
        printf("CRIT 5 %.17g\n", calc_logloss(&prob, model));
        printf("CRIT 6 %.17g\n", calc_accuracy(&prob, model));
        const int ids[4] = {10, 11, 12, 13};
        for (int c = 0; c < 4; ++c) {
            mf::mf_problem p2 = mf::read_problem(std::string(argv[1]));
            const bool transpose = (ids[c] == 11 || ids[c] == 13);
            const double v = ids[c] <= 11 ? calc_mpr(&p2, model, transpose) : calc_auc(&p2, model, transpose);
            printf("CRIT %d %.17g\n", ids[c], v);
        }
    }
    return 0;
}
