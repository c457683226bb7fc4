// mm_read.hpp -- minimal MatrixMarket reader for the command-line drivers:
// "coordinate" (real / integer / pattern; general / symmetric /
// skew-symmetric) into 0-based CSC with 64-bit indices, and "array" (real /
// integer, general) into a column-major dense buffer.  Duplicate coordinate
// entries are summed.  Throws std::runtime_error on malformed input.
#pragma once
#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

struct MMMatrix {
    int64_t m = 0, n = 0;
    bool dense = false;
    std::vector<int64_t> p, i;   // CSC (coordinate input)
    std::vector<double> x;       // CSC values, or the dense column-major buffer
};

inline std::string mm_lower(std::string s)
{
    for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
    return s;
}

inline MMMatrix mm_read(const std::string& path)
{
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open " + path);
    std::string line;
    if (!std::getline(in, line)) throw std::runtime_error("empty file " + path);
    std::istringstream hs(line);
    std::string banner, object, format, field, symmetry;
    hs >> banner >> object >> format >> field >> symmetry;
    if (mm_lower(banner) != "%%matrixmarket" || mm_lower(object) != "matrix")
        throw std::runtime_error("not a MatrixMarket matrix: " + path);
    format = mm_lower(format);
    field = mm_lower(field);
    symmetry = mm_lower(symmetry);
    if (field == "complex") throw std::runtime_error("complex matrices are not supported");
    const bool pattern = field == "pattern";
    const bool sym = symmetry == "symmetric", skew = symmetry == "skew-symmetric";
    while (std::getline(in, line))
        if (!line.empty() && line[0] != '%') break;
    std::istringstream ss(line);
    MMMatrix A;
    if (format == "array") {
        if (sym || skew) throw std::runtime_error("symmetric array format is not supported");
        ss >> A.m >> A.n;
        A.dense = true;
        A.x.resize((size_t)(A.m * A.n));
        for (int64_t e = 0; e < A.m * A.n; ++e)
            if (!(in >> A.x[(size_t)e])) throw std::runtime_error("truncated array data");
        return A;
    }
    if (format != "coordinate") throw std::runtime_error("unknown format " + format);
    int64_t nnz = 0;
    ss >> A.m >> A.n >> nnz;
    struct T3 { int64_t r, c; double v; };
    std::vector<T3> t;
    t.reserve((size_t)(sym || skew ? 2 * nnz : nnz));
    for (int64_t e = 0; e < nnz; ++e) {
        int64_t r, c;
        double v = 1.0;
        if (!(in >> r >> c)) throw std::runtime_error("truncated coordinate data");
        if (!pattern && !(in >> v)) throw std::runtime_error("truncated coordinate data");
        if (r < 1 || r > A.m || c < 1 || c > A.n) throw std::runtime_error("index out of range");
        t.push_back({r - 1, c - 1, v});
        if ((sym || skew) && r != c) t.push_back({c - 1, r - 1, skew ? -v : v});
    }
    std::sort(t.begin(), t.end(), [](const T3& a, const T3& b) {
        return a.c != b.c ? a.c < b.c : a.r < b.r;
    });
    A.p.assign((size_t)A.n + 1, 0);
    for (size_t q = 0; q < t.size(); ++q) {
        if (!A.i.empty() && q > 0 && t[q].c == t[q - 1].c && t[q].r == t[q - 1].r) {
            A.x.back() += t[q].v;   // duplicate entry
            continue;
        }
        A.i.push_back(t[q].r);
        A.x.push_back(t[q].v);
        A.p[(size_t)t[q].c + 1]++;
    }
    for (int64_t j = 0; j < A.n; ++j) A.p[(size_t)j + 1] += A.p[(size_t)j];
    return A;
}

// Transpose of a CSC matrix (m x n -> n x m), row indices kept sorted.
inline MMMatrix mm_transpose(const MMMatrix& A)
{
    MMMatrix B;
    B.m = A.n;
    B.n = A.m;
    B.p.assign((size_t)B.n + 1, 0);
    for (int64_t r : A.i) B.p[(size_t)r + 1]++;
    for (int64_t j = 0; j < B.n; ++j) B.p[(size_t)j + 1] += B.p[(size_t)j];
    B.i.resize(A.i.size());
    B.x.resize(A.x.size());
    std::vector<int64_t> pos(B.p.begin(), B.p.end() - 1);
    for (int64_t c = 0; c < A.n; ++c)
        for (int64_t q = A.p[(size_t)c]; q < A.p[(size_t)c + 1]; ++q) {
            const int64_t r = A.i[(size_t)q];
            B.i[(size_t)pos[(size_t)r]] = c;
            B.x[(size_t)pos[(size_t)r]++] = A.x[(size_t)q];
        }
    return B;
}
