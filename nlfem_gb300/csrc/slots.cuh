// CSR slot lookup and fixed-point accumulation for the one-sided pass.
//
// The pass adds every element pair's blocks into the rows of both elements (the reference adds
// termNonloc / termLocal into the outer element's rows and termNonlocPrime / termLocalPrime into
// the inner element's rows, Cassemble.cpp:737-766), from many warps at once. To keep the result
// independent of the order those additions land in, each contribution is first rounded to a
// 64-bit fixed-point integer (unit 2^fx_ue of its problem) and added with an integer atomic:
// integer addition is associative, so the sums are identical run to run.
//
// Slots are found without binary search, by one of two per-row maps from a column to its
// position in the sorted row:
//  * window rank (the default): the row's columns as a bitmap over the column range
//    [first, last] of the row, stored as 32-bit words with, beside each word, the count of the
//    row's columns in the earlier words; one 8-byte load finds a slot. Its size follows the
//    range of vertex numbers a row spans, so it is used when all rows together need at most
//    RANK_WORDS_PER_NNZ words per stored entry;
//  * hash (otherwise): an open-addressing table per row (capacity a power of two >= 2 x row
//    length, linear probing).
// tpos[s] gives, for the slot s = (i, j), the position of column i in row j (the pattern is
// symmetric on kept rows), and dslot lists the slots of each element's diagonal block.
#pragma once
#include "passes.cuh"

namespace nlg {

constexpr unsigned long long HEMPTY = ~0ULL;
constexpr int FX_GUARD = 10;   // bits of headroom above the problem's entry magnitude
constexpr int RANK_WORDS_PER_NNZ = 2;   // window-rank maps up to this many words per stored entry

struct SlotMap {
    const long long *rowptr;          // CSR row starts (rows of vertices with label <= 0 are empty)
    const long long *hptr;            // hash: per row, start of its table; capacity = hptr[u+1]-hptr[u]
    const unsigned long long *htab;   // hash: entries (position << 32) | column, HEMPTY when free
    const uint2 *rank;                // window rank (null: hash): per word {column bits, earlier columns}
    const long long *rbase;           // window rank: per row, first word; words = rbase[u+1] - rbase[u]
    const int *rlo;                   // window rank: per row, column >> 5 of its first word
    const int *tpos;                  // per slot (i, j): position of column i in row j, -1 if row j is empty
    const int *dslot;                 // per element: (dim+1)^2 slots of its diagonal block, -1 if the row is empty
};

// Slot of (u, col) in the window-rank map, or -1.
__device__ __forceinline__ long long rank_find(const SlotMap &m, int u, int col) {
    const long long b = m.rbase[u];
    const unsigned words = (unsigned)(m.rbase[u + 1] - b);
    const unsigned w = (unsigned)((col >> 5) - m.rlo[u]);
    if (w >= words) return -1;
    const uint2 e = m.rank[b + w];
    const unsigned bit = 1u << (col & 31);
    if (!(e.x & bit)) return -1;
    return m.rowptr[u] + (long long)e.y + __popc(e.x & (bit - 1u));
}

// Slot of (u, col), or -1 when the row has no such column. At most capacity probes.
__device__ __forceinline__ long long slot_find(const SlotMap &m, int u, int col) {
    if (m.rank) return rank_find(m, u, col);
    const long long hb = m.hptr[u];
    const unsigned cap = (unsigned)(m.hptr[u + 1] - hb);
    if (cap == 0) return -1;
    const unsigned mask = cap - 1;
    unsigned h = hash32((unsigned)col) & mask;
    for (unsigned probe = 0; probe < cap; probe++) {
        const unsigned long long e = m.htab[hb + h];
        if (e == HEMPTY) return -1;
        if ((unsigned)(e & 0xffffffffULL) == (unsigned)col) return m.rowptr[u] + (long long)(e >> 32);
        h = (h + 1) & mask;
    }
    return -1;
}

// The map of one row, loaded once for many lookups. Hash: hb the table start, mask = capacity - 1.
// Window rank: hb the first word, mask the word count, lo the first word's column >> 5. An empty
// row has mask 0xffffffff and never matches.
struct RowHash {
    long long hb, rb;   // map start, CSR row start
    unsigned mask;
    int lo;
};
__device__ __forceinline__ RowHash row_hash(const SlotMap &m, int u) {
    RowHash h;
    h.rb = m.rowptr[u];
    h.lo = 0;
    if (m.rank) {
        h.hb = m.rbase[u];
        const unsigned words = (unsigned)(m.rbase[u + 1] - h.hb);
        h.mask = words ? words : 0xffffffffu;
        h.lo = m.rlo[u];
        return h;
    }
    h.hb = m.hptr[u];
    const unsigned cap = (unsigned)(m.hptr[u + 1] - h.hb);
    h.mask = cap ? cap - 1 : 0xffffffffu;
    return h;
}

// A lookup in two halves, so that several lookups can have their first memory access in flight
// together: slot_probe_begin issues it (the rank word, or the first hash entry), slot_probe_end
// finishes the lookup (for the hash, with the rest of the probe sequence).
struct SlotProbe {
    unsigned long long e;
    unsigned i;
};
__device__ __forceinline__ SlotProbe slot_probe_begin(const SlotMap &m, const RowHash &h, int col) {
    SlotProbe p;
    p.e = HEMPTY;
    p.i = 0;
    if (h.mask == 0xffffffffu) return p;
    if (m.rank) {
        const unsigned w = (unsigned)((col >> 5) - h.lo);
        if (w < h.mask) {
            const uint2 r = m.rank[h.hb + w];
            p.e = ((unsigned long long)r.y << 32) | r.x;
            p.i = 1;
        }
        return p;
    }
    p.i = hash32((unsigned)col) & h.mask;
    p.e = m.htab[h.hb + p.i];
    return p;
}
__device__ __forceinline__ long long slot_probe_end(const SlotMap &m, const RowHash &h, int col, SlotProbe p) {
    if (h.mask == 0xffffffffu) return -1;
    if (m.rank) {
        const unsigned bits = (unsigned)p.e, bit = 1u << (col & 31);
        if (!p.i || !(bits & bit)) return -1;
        return h.rb + (long long)(p.e >> 32) + __popc(bits & (bit - 1u));
    }
    unsigned i = p.i;
    unsigned long long e = p.e;
    for (unsigned probe = 0; probe <= h.mask; probe++) {
        if (e == HEMPTY) return -1;
        if ((unsigned)(e & 0xffffffffULL) == (unsigned)col) return h.rb + (long long)(e >> 32);
        i = (i + 1) & h.mask;
        e = m.htab[h.hb + i];
    }
    return -1;
}

__device__ __forceinline__ long long slot_find_row(const SlotMap &m, const RowHash &h, int col) {
    if (h.mask == 0xffffffffu) return -1;
    if (m.rank) return slot_probe_end(m, h, col, slot_probe_begin(m, h, col));
    unsigned i = hash32((unsigned)col) & h.mask;
    for (unsigned probe = 0; probe <= h.mask; probe++) {
        const unsigned long long e = m.htab[h.hb + i];
        if (e == HEMPTY) return -1;
        if ((unsigned)(e & 0xffffffffULL) == (unsigned)col) return h.rb + (long long)(e >> 32);
        i = (i + 1) & h.mask;
    }
    return -1;
}

// Fixed-point value of a contribution: round(v * 2^-fx_ue); out of range (or not finite) sets
// the overflow flag, which makes the host redo the pass with a coarser unit.
__device__ __forceinline__ long long fx64(float v, float mul, int *ovf) {
    const float t = v * mul;
    if (!(fabsf(t) < 4.0e18f)) {
        atomicOr(ovf, 1);
        return 0;
    }
    return __float2ll_rn(t);
}
// The same with the overflow recorded in a flag of the caller (reported once, not per value).
__device__ __forceinline__ long long fx64(float v, float mul, bool &bad) {
    const float t = v * mul;
    const bool ok = fabsf(t) < 4.0e18f;
    bad |= !ok;
    return ok ? __float2ll_rn(t) : 0;
}
__device__ __forceinline__ long long fx64d(double v, double mul, bool &bad) {
    const double t = v * mul;
    const bool ok = fabs(t) < 4.0e18;
    bad |= !ok;
    return ok ? __double2ll_rn(t) : 0;
}
__device__ __forceinline__ long long fx64d(double v, double mul, int *ovf) {
    const double t = v * mul;
    if (!(fabs(t) < 4.0e18)) {
        atomicOr(ovf, 1);
        return 0;
    }
    return __double2ll_rn(t);
}
// Adds v to vals[s] (a zero is added too: a branch at every call site costs more than the
// reduction).
__device__ __forceinline__ void red_add(long long *vals, long long s, long long v) {
    atomicAdd(reinterpret_cast<unsigned long long *>(vals) + s, (unsigned long long)v);
}

// ------------------------------------------------------------------ construction
// Capacity of each row's table: the smallest power of two >= 2 x row length (0 for empty rows).
__global__ void k_hash_cap(const long long *__restrict__ rowptr, long long nV, long long *__restrict__ cap) {
    const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nV) return;
    const long long n = rowptr[u + 1] - rowptr[u];
    long long c = 0;
    if (n > 0) {
        c = 2;
        while (c < 2 * n) c <<= 1;
    }
    cap[u] = c;
}

// One warp per row: insert (position, column) of every slot. A free entry always exists within
// capacity probes (load factor <= 1/2).
__global__ void k_hash_fill(const long long *__restrict__ rowptr, const int *__restrict__ cols, long long nV,
                            const long long *__restrict__ hptr, unsigned long long *__restrict__ htab) {
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long u = gw; u < nV; u += nw) {
        const long long b = rowptr[u];
        const int n = (int)(rowptr[u + 1] - b);
        const long long hb = hptr[u];
        const unsigned cap = (unsigned)(hptr[u + 1] - hb);
        if (n == 0 || cap == 0) continue;
        const unsigned mask = cap - 1;
        for (int i = lane; i < n; i += 32) {
            const int col = cols[b + i];
            const unsigned long long e = ((unsigned long long)(unsigned)i << 32) | (unsigned)col;
            unsigned h = hash32((unsigned)col) & mask;
            for (unsigned probe = 0; probe < cap; probe++) {
                if (atomicCAS(&htab[hb + h], HEMPTY, e) == HEMPTY) break;
                h = (h + 1) & mask;
            }
        }
    }
}

// Window-rank map. k_rank_words: words of each row's window ((last >> 5) - (first >> 5) + 1, 0
// for an empty row) and the first word's index.
__global__ void k_rank_words(const long long *__restrict__ rowptr, const int *__restrict__ cols, long long nV,
                             long long *__restrict__ words, int *__restrict__ rlo) {
    const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nV) return;
    const long long b = rowptr[u], e = rowptr[u + 1];
    if (e == b) { words[u] = 0; rlo[u] = 0; return; }
    const int lo = cols[b] >> 5, hi = cols[e - 1] >> 5;   // rows are sorted
    words[u] = hi - lo + 1;
    rlo[u] = lo;
}

// One warp per row: the column bits of every word (each word's columns are a run of the sorted
// row; the lane holding a run's first column assembles the word), then the counts of earlier
// columns by a warp scan over the words.
__global__ void k_rank_fill(const long long *__restrict__ rowptr, const int *__restrict__ cols, long long nV,
                            const long long *__restrict__ rbase, const int *__restrict__ rlo,
                            uint2 *__restrict__ rank) {
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long u = gw; u < nV; u += nw) {
        const long long b = rowptr[u], n = rowptr[u + 1] - b;
        const long long wb = rbase[u];
        const int words = (int)(rbase[u + 1] - wb), lo = rlo[u];
        for (int w = lane; w < words; w += 32) rank[wb + w] = make_uint2(0u, 0u);
        __syncwarp();
        for (long long i = lane; i < n; i += 32) {
            const int c = cols[b + i];
            if (i > 0 && (cols[b + i - 1] >> 5) == (c >> 5)) continue;   // not the first of its word
            unsigned bits = 0;
            for (long long j = i; j < n && (cols[b + j] >> 5) == (c >> 5); j++) bits |= 1u << (cols[b + j] & 31);
            rank[wb + (c >> 5) - lo].x = bits;
        }
        __syncwarp();
        unsigned carry = 0;
        for (int w0 = 0; w0 < words; w0 += 32) {
            const int w = w0 + lane;
            const unsigned c = w < words ? (unsigned)__popc(rank[wb + w].x) : 0u;
            const unsigned incl = warp_incl_scan(c, lane);
            if (w < words) rank[wb + w].y = carry + incl - c;
            carry += __shfl_sync(FULL, incl, 31);
        }
        __syncwarp();
    }
}

// One warp per row i: tpos of each slot (i, j).
__global__ void k_tpos(SlotMap m, const int *__restrict__ cols, const int *__restrict__ labV, long long nV,
                       int *__restrict__ tpos, int *__restrict__ err) {
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = gw; i < nV; i += nw) {
        const long long b = m.rowptr[i], e = m.rowptr[i + 1];
        for (long long s = b + lane; s < e; s += 32) {
            const int j = cols[s];
            int p = -1;
            if (labV[j] > 0) {
                const long long t = slot_find(m, j, (int)i);
                if (t < 0) atomicOr(&err[3], 1);
                else p = (int)(t - m.rowptr[j]);
            }
            tpos[s] = p;
        }
    }
}

// Diagonal-block slots of every element (-1 where the row is empty or, for an element without
// any pair, where the pattern has no such slot).
template <int DIM>
__global__ void k_dslot(SlotMap m, const int *__restrict__ T32, const int *__restrict__ labV, long long nE,
                        int *__restrict__ dslot) {
    constexpr int dV = DIM + 1;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE) return;
#pragma unroll
    for (int r = 0; r < dV; r++) {
        const int u = T32[e * dV + r];
        const bool keep = labV[u] > 0;
#pragma unroll
        for (int c = 0; c < dV; c++)
            dslot[e * dV * dV + r * dV + c] = keep ? (int)slot_find(m, u, T32[e * dV + c]) : -1;
    }
}

}  // namespace nlg
