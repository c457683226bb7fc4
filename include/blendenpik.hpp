/*
 * blendenpik.hpp -- C++ drop-in for the reference's Blendenpik comparison
 * solver (include/blendenpik.hpp:31-33, src/ls_dense_blendenpik.cpp:21-70):
 * the same signature, implemented over skl_dense_blendenpik_solve.
 *
 * Sketch: random signs, orthonormal DHT of the columns (padded to a smooth
 * length with wisdom = 1), m = ceil(gamma*n) rows kept without replacement
 * (rand_subsampled_dct, src/dense_helpers.cpp:42-59); unpivoted QR of the
 * sample; LSQR preconditioned by R from x = 0; x = R^{-1} y; rank = n.  The
 * signs and the row draw each start from the stream reseeded with time(NULL),
 * as the reference's srand calls do.  A is left untouched.
 */
#ifndef SKILLS_BLENDENPIK_HPP
#define SKILLS_BLENDENPIK_HPP

#include "ski-lls.h"

inline void ls_dense_blendenpik(Mat_d& A, Vec_d& b, Vec_d& x, long& rank, int& flag, long& it,
                                double gamma, double it_tol, long max_it, int debug, int wisdom)
{
    (void)debug;
    if (A.m() != b.n() || A.n() != x.n() || b.inc() != 1 || x.inc() != 1)
        throw std::runtime_error("size mismatch");
    skl_opts o;
    skl_default_opts(&o);
    o.gamma = gamma;
    o.it_tol = it_tol;
    o.max_it = max_it;
    o.wisdom = wisdom;
    skl_info info;
    skills_gb300_detail::check(
        skl_dense_blendenpik_solve(A.data(), A.ld(), A.m(), A.n(), b.data(), x.data(), &o, &info));
    rank = (long)info.rank;
    flag = info.flag;
    it = (long)info.it;
}

#endif
