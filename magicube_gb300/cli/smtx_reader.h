// smtx_reader.h -- the .smtx reader of the benchmark programs.
//
// The reference's format (SpMM/SpMM/spmm_benchmark.cpp:126-175): a header
// line "rows, columns, nonzeros", then rows + 1 row offsets, then the column
// indices, whitespace separated.  Besides parsing, the reader checks what the
// packer relies on -- offsets start at 0, never decrease and end at the
// nonzero count, every column lies in [0, columns) -- so an inconsistent file
// is refused with a reason instead of being read past its arrays.
#pragma once
#include <climits>
#include <fstream>
#include <new>
#include <string>
#include <vector>

struct Smtx {
    int m_vec = 0, ncols = 0, nnz = 0;
    std::vector<int> offsets, cols;
};

// False, with the reason in `err`, for a missing, malformed or inconsistent file.
inline bool read_smtx(const std::string& path, Smtx& s, std::string& err)
{
    std::ifstream in(path);
    if (!in) {
        err = "cannot read " + path;
        return false;
    }
    long long head[3] = {0, 0, 0};
    try {
        std::string tok;
        for (int i = 0; i < 3; ++i) {
            if (!std::getline(in, tok, i < 2 ? ',' : '\n')) throw 0;
            head[i] = std::stoll(tok);
        }
    } catch (...) {
        err = path + ": malformed header (rows, columns, nonzeros)";
        return false;
    }
    if (head[0] < 0 || head[0] >= INT_MAX || head[1] <= 0 || head[1] > INT_MAX || head[2] < 0 || head[2] > INT_MAX) {
        err = path + ": header out of range";
        return false;
    }
    s.m_vec = (int)head[0];
    s.ncols = (int)head[1];
    s.nnz = (int)head[2];
    try {
        s.offsets.assign((size_t)s.m_vec + 1, 0);
        s.cols.assign((size_t)s.nnz, 0);
    } catch (const std::bad_alloc&) {
        err = path + ": too large to hold";
        return false;
    }
    for (auto& x : s.offsets) in >> x;
    for (auto& x : s.cols) in >> x;
    if (in.fail()) {
        err = path + ": fewer offsets or columns than the header declares";
        return false;
    }
    if (s.offsets[0] != 0 || s.offsets[(size_t)s.m_vec] != s.nnz) {
        err = path + ": row offsets must start at 0 and end at the nonzero count";
        return false;
    }
    for (int i = 0; i < s.m_vec; ++i)
        if (s.offsets[(size_t)i + 1] < s.offsets[(size_t)i]) {
            err = path + ": row offsets decrease";
            return false;
        }
    for (int c : s.cols)
        if (c < 0 || c >= s.ncols) {
            err = path + ": a column index lies outside [0, columns)";
            return false;
        }
    return true;
}
