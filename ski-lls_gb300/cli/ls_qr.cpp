// ls_qr -- command-line driver for ls_sparse_spqr on the GPU, with the
// argument order and printed lines of the reference's test/ls_qr.cpp:
//   argv[1] MatrixMarket file (sparse; a matrix with more columns than rows is
//           transposed), b = ones;
//   argv[2] over-sampling ratio gamma (1.4), argv[3] nnz per column k (2),
//   argv[4] absolute tolerance (ABS_TOL), argv[5] ordering (accepted; the GPU
//   path factorizes the sketch densely).
#include <cstdlib>
#include <iostream>

#include "ski-lls.h"
#include "mm_read.hpp"

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::cerr << "usage: ls_qr matrix.mtx [gamma] [k] [abs_tol] [ordering]" << std::endl;
        return 2;
    }
    std::cout.precision(PRINTING_PRECISION);
    std::cout << std::fixed;
    std::cout << std::endl << "==============BEGIN==================" << std::endl;
    std::cout << "Matrix path: " << argv[1] << std::endl;
    MMMatrix M;
    try {
        M = mm_read(argv[1]);
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
    if (M.dense) {
        std::cerr << "ls_qr expects a sparse (coordinate) matrix" << std::endl;
        return 1;
    }
    if (M.m < M.n) M = mm_transpose(M);
    std::cout << "number of rows is: " << M.m << std::endl;
    std::cout << "number of columns is: " << M.n << std::endl;
    std::cout << "number of non-zeros is: " << (long)M.x.size() << std::endl;
    cs_dl A{(int64_t)M.x.size(), M.m, M.n, M.p.data(), M.i.data(), M.x.data(), -1};
    double gamma = argc >= 3 ? std::atof(argv[2]) : 1.4;
    long k = argc >= 4 ? std::atol(argv[3]) : 2;
    double abs_tol = argc >= 5 ? std::atof(argv[4]) : ABS_TOL;
    int ordering = argc >= 6 ? std::atoi(argv[5]) : SPQR_ORDERING;
    std::cout << "Solver Name: Ls_qr" << std::endl;
    std::cout << "NNZ_PER_COLUMN is: " << k << std::endl;
    std::cout << "OVER_SAMPLING_RATIO is: " << gamma << std::endl;
    std::cout << "absolute tolerance is: " << abs_tol << std::endl;
    std::vector<double> ones((size_t)M.m, 1.0), xs((size_t)M.n, 0.0);
    Vec_d b(M.m, ones.data()), x(M.n, xs.data());
    long rank = 0, it = 0;
    int flag = 0;
    try {
        ls_sparse_spqr(A, b, x, rank, flag, it, gamma, k, abs_tol, ordering);
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
    std::cout << "Rank of A is: " << rank << std::endl;
    CSC_Mat_d Ac(M.m, M.n, (long)M.x.size(), (long*)M.i.data(), (long*)M.p.data(), M.x.data());
    Ac.mv('n', 1.0, x, -1.0, b);   // b <- A x - b
    std::cout << "Residual of ls_sparse_spqr is: " << nrm2(b) << std::endl;
    std::cout << "Iteration of ls_sparse_spqr is: " << it << std::endl;
    if (flag == 0) std::cout << "Status: LSQR Converged, a minimal residual solution found" << std::endl;
    else std::cout << "Status: Maximum iteration reached, a suboptimal solution found" << std::endl;
    std::cout << "==============FINISH==================" << std::endl << std::endl;
    return 0;
}
