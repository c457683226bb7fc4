// Sparse drop-in check: the CSC problem of the reference's sparse example
// (data from test/ski-llsSparseExample.cpp:11-13, :23) solved through ski-lls.h,
// plus the error path for a wide matrix.
#include <cstdio>
#include <stdexcept>
#include "ski-lls.h"

int main()
{
    long colp[4] = {0, 1, 3, 5};
    long rowi[5] = {0, 0, 2, 1, 3};
    double val[5] = {2.0, 3.0, 1.0, 4.0, 5.0};
    cs_dl* A = cs_dl_spalloc(4, 3, 5, 1, 0);
    std::free(A->p);
    std::free(A->i);
    std::free(A->x);
    A->p = colp;
    A->i = rowi;
    A->x = val;
    double rhs[4] = {0.0649338, 0.845946, -0.0164085, 0.247119};
    Vec_d b(4, rhs);
    Vec_d x(A->n);
    long rank = 0, it = 0;
    int flag = 0;
    ls_sparse_spqr(*A, b, x, rank, flag, it, OVER_SAMPLING_RATIO, NNZ_PER_COLUMN, ABS_TOL,
                   SPQR_ORDERING, IT_TOL, MAX_IT, RCOND_THRESHOLD, PERTURB, 0);
    CSC_Mat_d Acsc(A->m, A->n, A->nzmax, A->i, A->p, A->x);
    Vec_d r = b.copy();
    Acsc.mv('n', 1, x, -1, r);
    std::printf("x %.10f %.10f %.10f rank %ld flag %d it %ld residual %.10e\n", x(0), x(1), x(2),
                rank, flag, it, nrm2(r));
    cs_dl wide = *A;
    wide.m = 2;
    Vec_d b2(2, rhs);
    try {
        ls_sparse_spqr(wide, b2, x, rank, flag, it, 1.1, 1);
        std::printf("error-path: no exception\n");
    } catch (const std::runtime_error& e) {
        std::printf("error-path: %s\n", e.what());
    }
    std::free(A);
    return 0;
}
