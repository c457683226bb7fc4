// ls_blendenpik -- command-line driver for ls_dense_blendenpik (Blendenpik) on
// the GPU, with the argument order and printed lines of the reference's
// test/ls_blendenpik.cpp:
//   argv[1] MatrixMarket file (array or coordinate, densified), b = ones;
//   argv[2] over-sampling ratio gamma (2.2).
#include <cstdlib>
#include <iostream>

#include "ski-lls.h"
#include "blendenpik.hpp"
#include "mm_read.hpp"

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::cerr << "usage: ls_blendenpik matrix.mtx [gamma]" << std::endl;
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
    std::vector<double> dense;
    if (M.dense) {
        dense = M.x;
    } else {
        dense.assign((size_t)(M.m * M.n), 0.0);
        for (int64_t c = 0; c < M.n; ++c)
            for (int64_t q = M.p[(size_t)c]; q < M.p[(size_t)c + 1]; ++q)
                dense[(size_t)(M.i[(size_t)q] + c * M.m)] = M.x[(size_t)q];
    }
    std::cout << "number of rows is: " << M.m << std::endl;
    std::cout << "number of columns is: " << M.n << std::endl;
    Mat_d A(M.m, M.n, dense.data());
    double gamma = argc >= 3 ? std::atof(argv[2]) : 2.2;
    std::cout << "Solver Name: Ls_blendenpik" << std::endl;
    std::cout << "OVER_SAMPLING_RATIO is: " << gamma << std::endl;
    std::cout << "MAX_IT is: " << MAX_IT << std::endl;
    std::cout << "IT_TOL is: " << IT_TOL << std::endl;
    std::cout << "WISDOM is: " << WISDOM << std::endl;
    std::vector<double> ones((size_t)M.m, 1.0), xs((size_t)M.n, 0.0);
    Vec_d b(M.m, ones.data()), x(M.n, xs.data());
    long rank = 0, it = 0;
    int flag = 0;
    try {
        ls_dense_blendenpik(A, b, x, rank, flag, it, gamma, IT_TOL, MAX_IT, 0, WISDOM);
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
    std::cout << "Iteration flag is: " << flag << std::endl;
    A.mv('n', 1.0, x, -1.0, b);   // b <- A x - b
    std::cout << "Residual of ls_blendenpik is: " << nrm2(b) << std::endl;
    std::cout << "Iteration of ls_blendenpik is: " << it << std::endl;
    if (flag == 0) std::cout << "Status: LSQR Converged, a minimal residual solution found" << std::endl;
    else std::cout << "Status: Maximum iteration reached, a suboptimal solution found" << std::endl;
    std::cout << "==============FINISH==================" << std::endl << std::endl;
    return 0;
}
