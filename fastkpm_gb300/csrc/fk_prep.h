// fk_prep.h -- host preprocessing of a Hamiltonian for the device kernels, shared by
// the single engine (fk_engine.cu) and the batched engine (fk_batch.cu).
//
// Carries out set_H's scaling Hs = (H - avg I)/mag (reference src/engine_cpu.cpp:189-197,
// src/engine_cusparse.cpp:701-730), inserts a zero diagonal block in rows that store
// none, classifies every block (2: real multiple of the identity, 1: real entries,
// 0: general) and converts the entries to the engine precision.
#pragma once
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fastkpm_gb300.h"
#include "fk_dispatch.h"

namespace fk {

// row_ptr monotone from 0 to nnzb, columns in [0, n_b) and strictly increasing per row.
inline int check_bsr_pattern(int n_b, int nnzb, const int* row_ptr, const int* col_idx, std::string& why) {
    char buf[160];
    if (!row_ptr || (nnzb > 0 && !col_idx)) { why = "null pattern array"; return FK_ERR_ARG; }
    if (row_ptr[0] != 0 || row_ptr[n_b] != nnzb) { why = "row_ptr must run from 0 to nnzb"; return FK_ERR_PATTERN; }
    for (int i = 0; i < n_b; i++) {
        if (row_ptr[i + 1] < row_ptr[i]) {
            snprintf(buf, sizeof buf, "row_ptr decreases at row %d", i);
            why = buf;
            return FK_ERR_PATTERN;
        }
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) {
            if (col_idx[k] < 0 || col_idx[k] >= n_b) {
                snprintf(buf, sizeof buf, "column %d out of range in row %d", col_idx[k], i);
                why = buf;
                return FK_ERR_PATTERN;
            }
            if (k > row_ptr[i] && col_idx[k] <= col_idx[k - 1]) {
                snprintf(buf, sizeof buf, "columns not strictly increasing in row %d", i);
                why = buf;
                return FK_ERR_PATTERN;
            }
        }
    }
    return FK_OK;
}

struct PreparedH {
    std::vector<int> row_ptr;        // augmented, local (starts at 0)
    std::vector<int> col;            // augmented local block columns
    std::vector<unsigned> colc;      // (col + col_offset) | class << 30
    std::vector<unsigned char> hval; // entries in the engine precision
};

inline int prepare_H(int prec, int cplx, int n_b, int b, int nnzb, const int* row_ptr, const int* col_idx,
                     const double* val, double es_lo, double es_hi, int col_offset, PreparedH& out, std::string& why) {
    if (n_b <= 0 || nnzb < 0 || (!val && nnzb > 0)) { why = "bad sizes or null arrays"; return FK_ERR_ARG; }
    if (b != 1 && b != 2) { why = "block size must be 1 or 2"; return FK_ERR_UNSUPPORTED; }
    if (!(es_hi > es_lo)) { why = "energy scale needs hi > lo"; return FK_ERR_ARG; }
    int rc = check_bsr_pattern(n_b, nnzb, row_ptr, col_idx, why);
    if (rc != FK_OK) return rc;
    const int bb = b * b, cw = cplx ? 2 : 1;
    const double avg = (es_hi + es_lo) / 2.0, mag = (es_hi - es_lo) / 2.0;
    std::vector<double> hs;
    out.row_ptr.assign(n_b + 1, 0);
    out.col.clear();
    out.col.reserve((size_t)nnzb + n_b);
    hs.reserve(((size_t)nnzb + n_b) * bb * cw);
    for (int i = 0; i < n_b; i++) {
        bool diag_done = false;
        for (int k = row_ptr[i]; k <= row_ptr[i + 1]; k++) {
            const bool end = k == row_ptr[i + 1];
            const int j = end ? n_b : col_idx[k];
            if (!diag_done && j >= i) {
                out.col.push_back(i);
                const size_t base = hs.size();
                if (j == i) hs.insert(hs.end(), val + (size_t)k * bb * cw, val + (size_t)(k + 1) * bb * cw);
                else hs.insert(hs.end(), (size_t)bb * cw, 0.0);
                for (int q = 0; q < b; q++) hs[base + (size_t)(q * b + q) * cw] -= avg;
                diag_done = true;
                if (j == i) continue;
            }
            if (end) break;
            out.col.push_back(j);
            hs.insert(hs.end(), val + (size_t)k * bb * cw, val + (size_t)(k + 1) * bb * cw);
        }
        out.row_ptr[i + 1] = (int)out.col.size();
    }
    for (auto& v : hs) v /= mag;
    const int nk = (int)out.col.size();
    out.colc.resize(nk);
    for (int k = 0; k < nk; k++) {
        const double* v = &hs[(size_t)k * bb * cw];
        bool real = true, scal = true;
        for (int q = 0; q < bb; q++)
            if (cplx && v[q * cw + 1] != 0.0) real = false;
        for (int bj = 0; bj < b; bj++)
            for (int bi = 0; bi < b; bi++) {
                const double re = v[(bj * b + bi) * cw];
                if (bi != bj && re != 0.0) scal = false;
                if (bi == bj && re != v[0]) scal = false;
            }
        const unsigned cls = real ? (scal ? 2u : 1u) : 0u;
        out.colc[k] = (unsigned)(out.col[k] + col_offset) | (cls << 30);
    }
    const size_t nval = (size_t)nk * bb * cw;
    const size_t bytes = (size_t)nk * bb * elem_bytes(prec, cplx);
    out.hval.assign(bytes, 0);
    if (prec == kF64) {
        std::memcpy(out.hval.data(), hs.data(), sizeof(double) * nval);
    } else if (prec == kF32) {
        float* f = reinterpret_cast<float*>(out.hval.data());
        for (size_t q = 0; q < nval; q++) f[q] = (float)hs[q];
    } else {
        float* f = reinterpret_cast<float*>(out.hval.data());
        for (size_t q = 0; q < nval; q++) {
            const float hi = (float)hs[q];
            f[2 * q] = hi;
            f[2 * q + 1] = (float)(hs[q] - (double)hi);
        }
    }
    return FK_OK;
}

// Per-tile gather lists of the staged step kernel: for every tile of kThreads (row, lane)
// items, the distinct block columns its rows touch plus the tile's own rows, sorted; the
// slot of the tile's first own row; and for every H block the slot of its column.
struct TileTables {
    std::vector<int> uoff{0};             // tiles + 1 offsets into ucol
    std::vector<int> ucol;                // global block columns
    std::vector<int> own;                 // per tile
    std::vector<unsigned short> kslot;    // per H block (global block index)
    int umax = 0;
};

// Append one system's tiles. rp/col: the system's BSR (local rows, local columns); its
// blocks sit at global block index kslot_off + k and its columns at col_off + col.
inline bool append_tile_tables(const int* rp, const int* col, int n_b, int Gp, int col_off, size_t kslot_off,
                               TileTables& t) {
    const long long items = (long long)n_b * Gp;
    const long long tiles = (items + kThreads - 1) / kThreads;
    if (t.kslot.size() < kslot_off + (size_t)rp[n_b]) t.kslot.resize(kslot_off + (size_t)rp[n_b]);
    std::vector<int> u;
    for (long long tt = 0; tt < tiles; tt++) {
        const int r_lo = (int)(tt * kThreads / Gp);
        const long long tl = (tt + 1) * kThreads < items ? (tt + 1) * kThreads - 1 : items - 1;
        const int r_hi = (int)(tl / Gp);
        u.clear();
        for (int r = r_lo; r <= r_hi; r++) {
            u.push_back(r);
            for (int k = rp[r]; k < rp[r + 1]; k++) u.push_back(col[k]);
        }
        std::sort(u.begin(), u.end());
        u.erase(std::unique(u.begin(), u.end()), u.end());
        if (u.size() >= 65535) return false;
        t.own.push_back((int)(std::lower_bound(u.begin(), u.end(), r_lo) - u.begin()));
        for (int r = r_lo; r <= r_hi; r++)
            for (int k = rp[r]; k < rp[r + 1]; k++)
                t.kslot[kslot_off + k] = (unsigned short)(std::lower_bound(u.begin(), u.end(), col[k]) - u.begin());
        for (int c : u) t.ucol.push_back(c + col_off);
        t.uoff.push_back((int)t.ucol.size());
        if ((int)u.size() > t.umax) t.umax = (int)u.size();
    }
    return true;
}

// Largest number of H blocks one tile of kThreads (row, lane) items touches.
inline int max_tile_blocks(const int* row_ptr, int n_b, int Gp) {
    const long long items = (long long)n_b * Gp;
    const long long tiles = (items + kThreads - 1) / kThreads;
    int nk_max = 0;
    for (long long t = 0; t < tiles; t++) {
        const int r_lo = (int)(t * kThreads / Gp);
        const long long tl = (t + 1) * kThreads < items ? (t + 1) * kThreads - 1 : items - 1;
        const int r_hi = (int)(tl / Gp);
        const int nk = row_ptr[r_hi + 1] - row_ptr[r_lo];
        if (nk > nk_max) nk_max = nk;
    }
    return nk_max;
}

}  // namespace fk
