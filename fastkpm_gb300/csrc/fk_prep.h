// fk_prep.h -- host preprocessing of a Hamiltonian for the device kernels, shared by
// the single engine (fk_engine.cu) and the batched engine (fk_batch.cu).
//
// Carries out set_H's scaling Hs = (H - avg I)/mag (reference src/engine_cpu.cpp:53-61,
// src/engine_cusparse.cpp:701-730), inserts a zero diagonal block in rows that store
// none, classifies every block (2: real multiple of the identity, 1: real entries,
// 0: general) and converts the entries to the engine precision.
#pragma once
#include <algorithm>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/fastkpm_gb300.h"
#include "fk_dispatch.h"

namespace fk {

// Runs f(lo, hi) over [0, n) split into contiguous ranges on the host's cores (one range when
// n is small).
template <class F>
inline void parallel_ranges(int n, int min_range, F f) {
    unsigned nt = std::thread::hardware_concurrency();
    nt = std::max(1u, std::min(nt, 64u));
    const int parts = (int)std::min<long long>(nt, std::max<long long>(1, (long long)n / std::max(1, min_range)));
    if (parts <= 1) { f(0, n); return; }
    std::vector<std::thread> ts;
    ts.reserve(parts);
    for (int p = 0; p < parts; p++) {
        const int lo = (int)((long long)n * p / parts), hi = (int)((long long)n * (p + 1) / parts);
        ts.emplace_back(f, lo, hi);
    }
    for (auto& t : ts) t.join();
}

// row_ptr monotone from 0 to nnzb, columns in [0, n_b) and strictly increasing per row. The
// row_ptr pass runs first, so that no column is read through an out-of-range row bound; the
// column pass runs over row ranges in parallel and reports the first bad row.
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
    }
    std::mutex mu;
    int bad_row = n_b;
    parallel_ranges(n_b, 1 << 15, [&](int lo, int hi) {
        for (int i = lo; i < hi; i++) {
            for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) {
                if (col_idx[k] < 0 || col_idx[k] >= n_b || (k > row_ptr[i] && col_idx[k] <= col_idx[k - 1])) {
                    std::lock_guard<std::mutex> lk(mu);
                    if (i < bad_row) bad_row = i;
                    return;
                }
            }
        }
    });
    if (bad_row < n_b) {
        const int i = bad_row;
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) {
            if (col_idx[k] < 0 || col_idx[k] >= n_b) {
                snprintf(buf, sizeof buf, "column %d out of range in row %d", col_idx[k], i);
                break;
            }
            if (k > row_ptr[i] && col_idx[k] <= col_idx[k - 1]) {
                snprintf(buf, sizeof buf, "columns not strictly increasing in row %d", i);
                break;
            }
        }
        why = buf;
        return FK_ERR_PATTERN;
    }
    return FK_OK;
}

// Allocator whose resize leaves new elements uninitialised (the buffers below are written in
// full by prepare_H's parallel pass; zero-filling hundreds of MB first costs a serial pass).
template <class T>
struct UninitAlloc : std::allocator<T> {
    template <class U> struct rebind { using other = UninitAlloc<U>; };
    UninitAlloc() = default;
    template <class U> UninitAlloc(const UninitAlloc<U>&) {}
    template <class U> void construct(U* p) noexcept { ::new (static_cast<void*>(p)) U; }
    template <class U, class... A> void construct(U* p, A&&... a) { ::new (static_cast<void*>(p)) U(std::forward<A>(a)...); }
};

struct PreparedH {
    std::vector<int> row_ptr;                                    // augmented, local (starts at 0)
    std::vector<int> col;                                        // augmented local block columns
    std::vector<unsigned, UninitAlloc<unsigned>> colc;           // (col + col_offset) | class << 30
    std::vector<unsigned char, UninitAlloc<unsigned char>> hval; // entries in the engine precision
    std::vector<unsigned char> row_hsum;   // per row: 1 if its identity blocks (class 2, at least two) share one value
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
    // rows without a stored diagonal block get a zero one, at its sorted position
    out.row_ptr.assign(n_b + 1, 0);
    parallel_ranges(n_b, 1 << 15, [&](int lo, int hi) {
        for (int i = lo; i < hi; i++) {
            const int* c0 = col_idx + row_ptr[i];
            const int* c1 = col_idx + row_ptr[i + 1];
            const bool has_diag = std::binary_search(c0, c1, i);
            out.row_ptr[i + 1] = (int)(c1 - c0) + (has_diag ? 0 : 1);
        }
    });
    for (int i = 0; i < n_b; i++) out.row_ptr[i + 1] += out.row_ptr[i];
    const int nk = out.row_ptr[n_b];
    out.col.resize(nk);
    out.colc.resize(nk);
    const size_t ebytes = (size_t)elem_bytes(prec, cplx) / cw;   // bytes per real entry
    out.hval.resize((size_t)nk * bb * cw * ebytes);
    unsigned char* hv = out.hval.data();
    out.row_hsum.assign(n_b, 0);
    // every output block: Hs = (H - avg I) / mag in double, classified, converted to the
    // engine precision; each range of rows writes its own slice of the outputs
    parallel_ranges(n_b, 1 << 14, [&](int lo, int hi) {
        double v[8];
        for (int i = lo; i < hi; i++) {
            int kout = out.row_ptr[i];
            bool diag_done = false;
            int n_ident = 0;
            bool same_h = true;
            double h_ident = 0.0;
            for (int k = row_ptr[i]; k <= row_ptr[i + 1]; k++) {
                const bool end = k == row_ptr[i + 1];
                const int j = end ? n_b : col_idx[k];
                for (int pass = 0; pass < 2; pass++) {
                    // pass 0: the diagonal block (stored or inserted) when this column reaches it;
                    // pass 1: the stored block k
                    int jc;
                    const double* src;
                    if (pass == 0) {
                        if (diag_done || j < i) continue;
                        jc = i;
                        src = j == i ? val + (size_t)k * bb * cw : nullptr;
                        diag_done = true;
                    } else {
                        if (end || j == i) continue;
                        jc = j;
                        src = val + (size_t)k * bb * cw;
                    }
                    for (int q = 0; q < bb * cw; q++) v[q] = src ? src[q] : 0.0;
                    if (jc == i)
                        for (int q = 0; q < b; q++) v[(size_t)(q * b + q) * cw] -= avg;
                    for (int q = 0; q < bb * cw; q++) v[q] /= mag;
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
                    if (cls == 2u) {
                        if (n_ident++ == 0) h_ident = v[0];
                        else if (v[0] != h_ident) same_h = false;
                    }
                    out.col[kout] = jc;
                    out.colc[kout] = (unsigned)(jc + col_offset) | (cls << 30);
                    const size_t base = (size_t)kout * bb * cw;
                    if (prec == kF64) {
                        std::memcpy(hv + base * sizeof(double), v, sizeof(double) * bb * cw);
                    } else if (prec == kF32) {
                        float* f = reinterpret_cast<float*>(hv) + base;
                        for (int q = 0; q < bb * cw; q++) f[q] = (float)v[q];
                    } else {
                        float* f = reinterpret_cast<float*>(hv) + 2 * base;
                        for (int q = 0; q < bb * cw; q++) {
                            const float hi32 = (float)v[q];
                            f[2 * q] = hi32;
                            f[2 * q + 1] = (float)(v[q] - (double)hi32);
                        }
                    }
                    kout++;
                }
                if (end) break;
            }
            out.row_hsum[i] = (n_ident >= 2 && same_h) ? 1 : 0;
        }
    });
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
// Most blocks in one block row.
inline int max_row_blocks(const int* row_ptr, int n_b) {
    int m = 0;
    for (int i = 0; i < n_b; i++) m = row_ptr[i + 1] - row_ptr[i] > m ? row_ptr[i + 1] - row_ptr[i] : m;
    return m;
}
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
