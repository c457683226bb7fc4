// Dense drop-in check: the problem of the reference's dense example
// (data from test/ski-llsDenseExample.cpp:9-12) solved through ski-lls.h.
// Prints the solution, rank, flag and iterations on one line.
#include <cstdio>
#include "ski-lls.h"
#include "blendenpik.hpp"

int main()
{
    double a[8] = {0.306051, -1.53078, 1.64493, -1.61322, -0.2829, 0.474476, -0.586278, -0.610202};
    double rhs[4] = {0.0649338, 0.845946, -0.0164085, 0.247119};
    Mat_d A(4, 2, a);
    Vec_d b(4, rhs);
    Vec_d x(A.n());
    long rank = 0, it = 0;
    int flag = 0;
    ls_dense_hashing_blendenpik(A, b, x, rank, flag, it, OVER_SAMPLING_RATIO, NNZ_PER_COLUMN, ABS_TOL,
                                RCOND, IT_TOL, MAX_IT, 0, WISDOM);
    Vec_d r = b.copy();
    A.mv('n', 1, x, -1, r);
    std::printf("x %.10f %.10f rank %ld flag %d it %ld residual %.10e\n", x(0), x(1), rank, flag, it,
                nrm2(r));
    long rank2 = 0, it2 = 0;
    int flag2 = 0;
    Vec_d x2(A.n());
    ls_dense_hashing_blendenpik_noCPQR(A, b, x2, rank2, flag2, it2, 1.7, 1, 1e-12, MAX_IT, 0, WISDOM);
    std::printf("x2 %.10f %.10f rank %ld\n", x2(0), x2(1), rank2);
    // Blendenpik (include/blendenpik.hpp:31-33): 3 of the 4 transformed rows
    long rank3 = 0, it3 = 0;
    int flag3 = 0;
    Vec_d x3(A.n());
    ls_dense_blendenpik(A, b, x3, rank3, flag3, it3, 1.5, 1e-12, MAX_IT, 0, WISDOM);
    std::printf("x3 %.10f %.10f rank %ld\n", x3(0), x3(1), rank3);
    return 0;
}
