// Merge-path row reduction over a CSR-shaped adjacency (ptr[n+1], col[m]).
//
// Rows and entries are merged into one sequence of n+m items (a row's end
// follows its last entry); each CTA takes a fixed window of `T*IPT` items, so
// work is balanced whatever the degree skew (RMAT hubs with 10^5..10^6
// entries are spread over many CTAs; runs of empty rows cost one item each).
// The windows' start coordinates are precomputed once per graph (schedule).
//
// Inside a CTA: row ends and entry values (gathered through col) are staged in
// shared memory with coalesced 128-bit loads of col; every thread then walks
// IPT consecutive items sequentially.  A row split between threads is summed
// with a segmented scan over the threads' open-row partials (warp shuffles,
// then across warps); a row split between CTAs is finished by a fix-up kernel
// whose warps add the preceding CTAs' partials 32 at a time.  All reduction
// orders are fixed, so results are deterministic.  Completed rows are written
// out by all threads in row order (coalesced).
//
// The Op supplies: value type V, accumulator A,
//   V gather(j, u)            value of entry j whose column is u
//   A zero(), A add(A, V), A merge(A left, A right)
//   float2 emit(row, A)       finishes a row; the two partials it returns
//                             (PageRank: |change|, dangling mass) are summed
//                             per thread as fp32 TwoSum pairs (eg_red2), then
//                             per CTA in FP64, when REDUCE is set
#pragma once
#include "eg_internal.cuh"

#define EG_MP_NONE 0xffffffffu

template <class A>
struct eg_mp_carry {
    uint32_t head_row;  // row finished in this CTA that began in an earlier CTA
    uint32_t tail_row;  // row still open at the CTA's end (n if none)
    A head_val;         // this CTA's partial of head_row
    A tail_val;         // this CTA's partial of tail_row
};


// Warp shuffles for the accumulator types (float, float2, double, uint32_t).
template <class A>
__device__ __forceinline__ A eg_shfl_up(A v, int off) {
    return __shfl_up_sync(EG_FULL_MASK, v, off);
}
template <>
__device__ __forceinline__ float2 eg_shfl_up<float2>(float2 v, int off) {
    return make_float2(__shfl_up_sync(EG_FULL_MASK, v.x, off), __shfl_up_sync(EG_FULL_MASK, v.y, off));
}
template <class A>
__device__ __forceinline__ A eg_shfl_down(A v, int off) {
    return __shfl_down_sync(EG_FULL_MASK, v, off);
}
template <>
__device__ __forceinline__ float2 eg_shfl_down<float2>(float2 v, int off) {
    return make_float2(__shfl_down_sync(EG_FULL_MASK, v.x, off), __shfl_down_sync(EG_FULL_MASK, v.y, off));
}
template <class A>
__device__ __forceinline__ A eg_shfl_idx(A v, int src) {
    return __shfl_sync(EG_FULL_MASK, v, src);
}
template <>
__device__ __forceinline__ float2 eg_shfl_idx<float2>(float2 v, int src) {
    return make_float2(__shfl_sync(EG_FULL_MASK, v.x, src), __shfl_sync(EG_FULL_MASK, v.y, src));
}

__global__ void k_mp_schedule(const uint32_t *__restrict__ ptr, uint32_t n, uint32_t m, uint32_t items,
                              uint32_t ntiles, uint2 *__restrict__ coord);

template <int T, int IPT, class V, class A>
struct eg_mp_smem {
    static constexpr int W = T * IPT;
    static constexpr size_t rowend_off = 0;
    static constexpr size_t val_off = ((W + 2) * 4 + 15) & ~(size_t)15;
    static constexpr size_t sum_off = (val_off + W * sizeof(V) + 15) & ~(size_t)15;
    static constexpr size_t cval_off = (sum_off + W * sizeof(A) + 15) & ~(size_t)15;
    static constexpr size_t crow_off = (cval_off + T * sizeof(A) + 15) & ~(size_t)15;
    static constexpr size_t bytes = (crow_off + T * 4 + 15) & ~(size_t)15;
};

template <class Op, int T, int IPT, bool REDUCE>
__global__ void __launch_bounds__(T) k_mp_rows(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ col,
                                               uint32_t n, const uint2 *__restrict__ coord,
                                               eg_mp_carry<typename Op::A> *__restrict__ carry,
                                               double2 *__restrict__ part, Op op) {
    using V = typename Op::V;
    using A = typename Op::A;
    using L = eg_mp_smem<T, IPT, V, A>;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *s_rowend = (uint32_t *)(smem + L::rowend_off);
    V *s_val = (V *)(smem + L::val_off);
    A *s_sum = (A *)(smem + L::sum_off);
    A *s_cval = (A *)(smem + L::cval_off);
    uint32_t *s_crow = (uint32_t *)(smem + L::crow_off);
    __shared__ uint32_t s_head;
    __shared__ A s_headval;
    __shared__ double2 s_red[T / 32];
    __shared__ uint32_t s_wkey[T / 32], s_wfirst[T / 32];
    __shared__ A s_wval[T / 32];

    if (!op.active()) return;
    op.setup();
    const uint32_t tid = threadIdx.x;
    const uint32_t c = blockIdx.x;
    const uint2 c0 = coord[c], c1 = coord[c + 1];
    const uint32_t i0 = c0.x, j0 = c0.y;
    const uint32_t nrows = c1.x - i0, nedges = c1.y - j0;
    const uint32_t rs0 = ptr[i0];  // ptr has n+1 entries; i0 <= n
    if (tid == 0) s_head = EG_MP_NONE;

    // stage row ends (relative to j0); the open row nrows gets its end too
    for (uint32_t k = tid; k <= nrows; k += T) s_rowend[k] = (i0 + k < n) ? __ldg(ptr + i0 + k + 1) - j0 : 0xffffffffu;
    // stage entry values: scalar head to a 16-byte boundary, uint4 body, tail
    {
        const uint32_t head = min((4u - (j0 & 3u)) & 3u, nedges);
        if (tid < head) s_val[tid] = op.gather(j0 + tid, __ldg(col + j0 + tid));
        const uint32_t nvec = (nedges - head) >> 2;
        const uint4 *cv = reinterpret_cast<const uint4 *>(col + j0 + head);
        for (uint32_t k = tid; k < nvec; k += T) {
            uint4 q = __ldg(cv + k);
            uint32_t b = head + 4 * k;
            V a0 = op.gather(j0 + b, q.x), a1 = op.gather(j0 + b + 1, q.y);
            V a2 = op.gather(j0 + b + 2, q.z), a3 = op.gather(j0 + b + 3, q.w);
            s_val[b] = a0;
            s_val[b + 1] = a1;
            s_val[b + 2] = a2;
            s_val[b + 3] = a3;
        }
        for (uint32_t k = head + 4 * nvec + tid; k < nedges; k += T) s_val[k] = op.gather(j0 + k, __ldg(col + j0 + k));
    }
    __syncthreads();

    // merge-path search for this thread's first item
    const uint32_t total = nrows + nedges;
    const uint32_t d0 = min(tid * IPT, total), d1 = min(d0 + IPT, total);
    uint32_t lo = d0 > nedges ? d0 - nedges : 0, hi = min(d0, nrows);
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (s_rowend[mid] <= d0 - mid - 1) lo = mid + 1;
        else hi = mid;
    }
    uint32_t it = lo, jt = d0 - lo;
    const uint32_t it_start = it;
    // does this thread's first row begin before its first entry?
    const bool start_cont = (it == 0) ? (rs0 < j0 + jt) : (s_rowend[it - 1] < jt);
    A acc = op.zero();
    A first_part = op.zero();
    uint32_t first_row = EG_MP_NONE;
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        if (d0 + k < d1) {
            if (s_rowend[it] <= jt) {
                if (it == it_start && start_cont) {
                    first_part = acc;
                    first_row = it;
                } else {
                    s_sum[it] = acc;
                }
                acc = op.zero();
                it++;
            } else {
                acc = op.add(acc, s_val[jt]);
                jt++;
            }
        }
    }
    // Segmented inclusive scan of the threads' open-row partials, keyed by the
    // open row (keys never decrease with the thread index, so equal keys form
    // one run).  Fixed shuffle order: deterministic.
    const uint32_t lane = tid & 31, warp = tid >> 5;
    A v = acc;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const A pv = eg_shfl_up(v, off);
        const uint32_t pk = __shfl_up_sync(EG_FULL_MASK, it, off);
        if (lane >= (uint32_t)off && pk == it) v = op.merge(pv, v);
    }
    const uint32_t first_key = __shfl_sync(EG_FULL_MASK, it, 0);
    if (lane == 31) {
        s_wkey[warp] = it;
        s_wval[warp] = v;
        s_wfirst[warp] = first_key;
    }
    __syncthreads();
    {
        A ext = op.zero();
        bool has = false;
        for (int w2 = (int)warp - 1; w2 >= 0; w2--) {
            if (s_wkey[w2] != it) break;
            ext = has ? op.merge(s_wval[w2], ext) : s_wval[w2];
            has = true;
            if (s_wfirst[w2] != it) break;
        }
        if (has) v = op.merge(ext, v);
    }
    s_crow[tid] = it;
    s_cval[tid] = v;
    __syncthreads();

    // finish this thread's first row if earlier threads hold parts of it; a
    // row that began before the CTA is finished by the fix-up kernel
    if (first_row != EG_MP_NONE) {
        A tot = first_part;
        if (tid > 0 && s_crow[tid - 1] == first_row) tot = op.merge(s_cval[tid - 1], tot);
        if (first_row == 0 && rs0 < j0) {
            s_head = 0;
            s_headval = tot;
        } else {
            s_sum[first_row] = tot;
        }
    }
    if (tid == T - 1) {
        carry[c].tail_row = i0 + nrows;
        carry[c].tail_val = v;
    }
    __syncthreads();
    if (tid == 0) {
        carry[c].head_row = s_head == EG_MP_NONE ? EG_MP_NONE : i0;
        if (s_head != EG_MP_NONE) carry[c].head_val = s_headval;
    }
    // write out completed rows in order
    eg_red2 redf;
    const uint32_t r0 = (s_head != EG_MP_NONE) ? 1u : 0u;
    for (uint32_t r = r0 + tid; r < nrows; r += T) {
        const float2 x = op.emit(i0 + r, s_sum[r]);
        if (REDUCE) redf.add(x);
    }
    if (REDUCE) {
        double2 red = redf.wide();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            red.x += __shfl_down_sync(EG_FULL_MASK, red.x, o);
            red.y += __shfl_down_sync(EG_FULL_MASK, red.y, o);
        }
        if ((tid & 31) == 0) s_red[tid >> 5] = red;
        __syncthreads();
        if (tid == 0) {
            double2 s = make_double2(0.0, 0.0);
            for (int w = 0; w < T / 32; w++) {
                s.x += s_red[w].x;
                s.y += s_red[w].y;
            }
            part[c] = s;
        }
    }
}

// One warp per CTA with a head row: completes rows that span CTAs by adding
// the tail partials of the preceding CTAs, 32 CTAs per step (lanes in CTA
// order, a fixed shuffle tree: deterministic).
template <class Op, bool REDUCE>
__global__ void k_mp_fixup(const uint32_t *__restrict__ ptr, const uint2 *__restrict__ coord, uint32_t ntiles,
                           const eg_mp_carry<typename Op::A> *__restrict__ carry, double2 *__restrict__ part, Op op) {
    using A = typename Op::A;
    __shared__ double2 s_red[32];
    if (!op.active()) return;
    op.setup();
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    eg_red2 redf;
    if (c < ntiles) {
        const uint32_t row = carry[c].head_row;
        if (row != EG_MP_NONE) {
            A tot = carry[c].head_val;
            const uint32_t rstart = ptr[row];
            for (int base = (int)c - 1; base >= 0; base -= 32) {
                const int k = base - (int)lane;
                const bool valid = k >= 0;
                const bool began = valid && rstart >= coord[k].y;  // the row begins inside CTA k
                const uint32_t stop_mask = __ballot_sync(EG_FULL_MASK, began || !valid);
                const int last = stop_mask ? __ffs(stop_mask) - 1 : 31;  // lanes 0..last contribute
                A x = (valid && (int)lane <= last) ? carry[k].tail_val : op.zero();
                // reduce lanes 0..31 (zeros past `last`) in a fixed tree, far-to-near order
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const A y = eg_shfl_down(x, off);
                    x = op.merge(y, x);
                }
                x = eg_shfl_idx(x, 0);
                tot = op.merge(x, tot);
                if (stop_mask) break;
            }
            if (lane == 0) redf.add(op.emit(row, tot));
        }
    }
    if (REDUCE) {
        if (lane == 0) s_red[threadIdx.x >> 5] = redf.wide();
        __syncthreads();
        if (threadIdx.x == 0) {
            double2 s = make_double2(0.0, 0.0);
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
                s.x += s_red[w].x;
                s.y += s_red[w].y;
            }
            part[blockIdx.x] = s;
        }
    }
}

// Compensated summation (Knuth's TwoSum) on fp32 pairs (sum, error).
struct eg_f2sum {
    __device__ __forceinline__ static float2 add(float2 a, float x) {
        float s = __fadd_rn(a.x, x);
        float bb = __fsub_rn(s, a.x);
        float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(x, bb));
        return make_float2(s, __fadd_rn(a.y, err));
    }
    __device__ __forceinline__ static float2 merge(float2 a, float2 b) {
        float2 r = add(a, b.x);
        r.y = __fadd_rn(r.y, b.y);
        return r;
    }
};

// ============================================================== row-id stream variant
// Entries carry their row id (rid[e], the COO form of the CSR/CSC, built once
// per graph), so a warp can own a fixed range of entries and find row
// boundaries by comparing neighbouring row ids.  Rows split between warps are
// finished by k_coo_fixup (same head/tail scheme as the merge-path kernels);
// rows without entries are written by k_coo_empty_rows (or, when they are
// known to form the range at the end, k_coo_empty_range).

// The block's share of the emitted (residual, dangling) partials into part[blockIdx.x].
template <bool REDUCE>
__device__ __forceinline__ void eg_block_part(const eg_red2 &redf, double2 *__restrict__ part, double2 *s_red) {
    if (!REDUCE) return;
    double2 red = redf.wide();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        red.x += __shfl_down_sync(EG_FULL_MASK, red.x, o);
        red.y += __shfl_down_sync(EG_FULL_MASK, red.y, o);
    }
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = red;
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 t = make_double2(0.0, 0.0);
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            t.x += s_red[w].x;
            t.y += s_red[w].y;
        }
        part[blockIdx.x] = t;
    }
}

// Rows split between warp tiles, finished from the tiles' head and tail
// partials: one thread per tile.  A head row that began in the tile before
// is finished by the tile's thread (that tile's tail + this tile's head);
// a row spanning more tiles is finished by the whole warp, which adds the
// tails of the preceding tiles 32 per step.  Both give the same bits (the
// tail and head are merged in that order either way).
template <class Op, int TILE_E, bool REDUCE>
__global__ void k_coo_fixup(const uint32_t *__restrict__ ptr, uint32_t ntiles,
                            const eg_mp_carry<typename Op::A> *__restrict__ carry, double2 *__restrict__ part,
                            Op op) {
    using A = typename Op::A;
    __shared__ double2 s_red[32];
    if (!op.active()) return;
    op.setup();
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    eg_red2 redf;
    uint32_t row = EG_MP_NONE, rstart = 0;
    bool wide = false;
    if (c < ntiles) {
        row = carry[c].head_row;  // never set in tile 0
        if (row != EG_MP_NONE) {
            rstart = ptr[row];
            if (c >= 1 && rstart >= (c - 1) * (uint32_t)TILE_E) {
                const float2 d = op.emit(row, op.merge(carry[c - 1].tail_val, carry[c].head_val));
                if (REDUCE) redf.add(d);
            } else {
                wide = true;
            }
        }
    }
    uint32_t todo = __ballot_sync(EG_FULL_MASK, wide);
    while (todo) {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1;
        const uint32_t cw = __shfl_sync(EG_FULL_MASK, c, src);
        const uint32_t rw = __shfl_sync(EG_FULL_MASK, row, src);
        const uint32_t sw = __shfl_sync(EG_FULL_MASK, rstart, src);
        A tot = carry[cw].head_val;
        for (int base = (int)cw - 1; base >= 0; base -= 32) {
            const int k = base - (int)lane;
            const bool valid = k >= 0;
            const bool began = valid && sw >= (uint32_t)k * (uint32_t)TILE_E;
            const uint32_t stop_mask = __ballot_sync(EG_FULL_MASK, began || !valid);
            const int last = stop_mask ? __ffs(stop_mask) - 1 : 31;
            A x = (valid && (int)lane <= last) ? carry[k].tail_val : op.zero();
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const A y = eg_shfl_down(x, off);
                x = op.merge(y, x);
            }
            x = eg_shfl_idx(x, 0);
            tot = op.merge(x, tot);
            if (stop_mask) break;
        }
        if ((int)lane == src) {
            const float2 d = op.emit(rw, tot);
            if (REDUCE) redf.add(d);
        }
    }
    eg_block_part<REDUCE>(redf, part, s_red);
}

// Rows without entries: emitted with an empty sum.  Four rows per thread and
// step, their row pointers loaded before any is tested.
template <class Op, bool REDUCE>
__global__ void k_coo_empty_rows(const uint32_t *__restrict__ ptr, uint32_t n, double2 *__restrict__ part, Op op) {
    __shared__ double2 s_red[32];
    if (!op.active()) return;
    op.setup();
    eg_red2 redf;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t v0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v0 < n; v0 += 4 * stride) {
        uint32_t lo[4], hi[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const uint64_t v = v0 + j * stride;
            lo[j] = 0;
            hi[j] = 1;
            if (v < n) {
                lo[j] = __ldg(ptr + v);
                hi[j] = __ldg(ptr + v + 1);
            }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (lo[j] == hi[j]) {
                const float2 d = op.emit((uint32_t)(v0 + j * stride), op.zero());
                if (REDUCE) redf.add(d);
            }
        }
    }
    eg_block_part<REDUCE>(redf, part, s_red);
}

// Rows [lo, hi), known to have no entries (the relabelled CSC keeps them
// last): emitted with an empty sum, without reading row pointers.
template <class Op, bool REDUCE>
__global__ void k_coo_empty_range(uint32_t lo, uint32_t hi, double2 *__restrict__ part, Op op) {
    __shared__ double2 s_red[32];
    if (!op.active()) return;
    op.setup();
    eg_red2 redf;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t v = (uint64_t)lo + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < hi; v += stride) {
        const float2 d = op.emit((uint32_t)v, op.zero());
        if (REDUCE) redf.add(d);
    }
    eg_block_part<REDUCE>(redf, part, s_red);
}

// 128-bit streaming load of the row-id / column words.  HINT 1: the words
// are not kept in L1 and are the first evicted from L2, which leaves both
// caches to the gathered vector (the words are read once per pass).
template <int HINT>
__device__ __forceinline__ uint4 eg_stream_ld4(const uint32_t *p, uint64_t pol) {
    if constexpr (HINT == 0) {
        return __ldg(reinterpret_cast<const uint4 *>(p));
    } else {
        uint4 v;
        asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
            : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
            : "l"(p), "l"(pol));
        return v;
    }
}

// One streamed 4-byte value (read once per pass): not kept in L1, first in
// line for L2 eviction, so the caches stay with the gathered vector.
__device__ __forceinline__ float eg_stream_ldf(const float *p, uint64_t pol) {
    float v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ uint64_t eg_l2_evict_first_policy() {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// The chunk of a warp tile starting at cb: lane l's entries cb+U*l ..
// cb+U*l+U-1 (128-bit loads), rows past the tile end E1 set to EG_MP_NONE.
template <int U, int HINT = 0>
__device__ __forceinline__ void eg_coov_load(const uint32_t *__restrict__ rid, const uint32_t *__restrict__ col,
                                             uint32_t cb, uint32_t E1, uint32_t lane, uint32_t (&r)[U],
                                             uint32_t (&u)[U], uint64_t pol = 0) {
    const uint32_t e = cb + U * lane;
    if (e + U - 1 < E1) {
#pragma unroll
        for (int h = 0; h < U / 4; h++) {
            const uint4 rr = eg_stream_ld4<HINT>(rid + e + 4 * h, pol);
            const uint4 cc = eg_stream_ld4<HINT>(col + e + 4 * h, pol);
            r[4 * h] = rr.x; r[4 * h + 1] = rr.y; r[4 * h + 2] = rr.z; r[4 * h + 3] = rr.w;
            u[4 * h] = cc.x; u[4 * h + 1] = cc.y; u[4 * h + 2] = cc.z; u[4 * h + 3] = cc.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < U; k++) {
            const bool in = e + k < E1;
            r[k] = in ? __ldg(rid + e + k) : EG_MP_NONE;
            u[k] = in ? __ldg(col + e + k) : 0u;
        }
    }
}

// Block sum of the emitted (residual, dangling) pairs into part[blockIdx.x].
__device__ __forceinline__ void eg_coov_reduce(const eg_red2 &redf, double2 *s_red, uint32_t nwarps,
                                               double2 *__restrict__ part) {
    double2 red = redf.wide();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        red.x += __shfl_down_sync(EG_FULL_MASK, red.x, o);
        red.y += __shfl_down_sync(EG_FULL_MASK, red.y, o);
    }
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = red;
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 sum = make_double2(0.0, 0.0);
        for (uint32_t w = 0; w < nwarps; w++) {
            sum.x += s_red[w].x;
            sum.y += s_red[w].y;
        }
        part[blockIdx.x] = sum;
    }
}

// Masked form of the row-id stream: the rows of lane l's entries base+U*l ..
// base+U*l+U-1 from the row-start bits (one word per lane, bits U*l..U*l+U-1
// of the chunk's U words) and `rbefore`, the row of the entry before the
// chunk.  Valid when every row between the first and the last has entries,
// so that a row start always means the next row.  Entries past E1 get
// EG_MP_NONE.
template <int U>
__device__ __forceinline__ void eg_mask_rows(uint32_t mw, uint32_t lane, uint32_t base, uint32_t E1, uint32_t rbefore,
                                             uint32_t (&r)[U]) {
    const uint32_t bits = (mw >> ((U * lane) & 31)) & ((1u << U) - 1u);
    const uint32_t c = __popc(bits);
    uint32_t incl = c;  // starts up to this lane's last entry, within the chunk
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(EG_FULL_MASK, incl, off);
        if (lane >= (uint32_t)off) incl += y;
    }
    const uint32_t r0 = rbefore + (incl - c);
    const uint32_t e = base + U * lane;
#pragma unroll
    for (int k = 0; k < U; k++) r[k] = e + k < E1 ? r0 + __popc(bits & ((2u << k) - 1u)) : EG_MP_NONE;
}

// The columns of a chunk (as eg_coov_load) and, masked, the lane's row-start word.
template <int U, int HINT>
__device__ __forceinline__ void eg_coom_load(const uint32_t *__restrict__ col, const uint32_t *__restrict__ starts,
                                             uint32_t cb, uint32_t E1, uint32_t lane, uint32_t &mw,
                                             uint32_t (&u)[U], uint64_t pol) {
    const uint32_t e = cb + U * lane;
    mw = e < E1 ? __ldg(starts + (e >> 5)) : 0u;  // lanes past the last entry read nothing
    if (e + U - 1 < E1) {
#pragma unroll
        for (int h = 0; h < U / 4; h++) {
            const uint4 cc = eg_stream_ld4<HINT>(col + e + 4 * h, pol);
            u[4 * h] = cc.x; u[4 * h + 1] = cc.y; u[4 * h + 2] = cc.z; u[4 * h + 3] = cc.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < U; k++) u[k] = e + k < E1 ? __ldg(col + e + k) : 0u;
    }
}

// One warp tile t of the row-id stream (the body of k_coov_rows);
// `gather(e, u)` returns the value of entry e, source u.  MK: rows from the
// row-start bits `starts` and the row of every EG_TROW_SPAN-th entry `trow`
// instead of the row ids (rid unused).
template <class Op, int TILE_E, int U, bool REDUCE, int PF, int HINT, bool MK, class G>
__device__ __forceinline__ void eg_coov_tile(uint32_t t, const uint32_t *__restrict__ rid,
                                             const uint32_t *__restrict__ col, const uint32_t *__restrict__ starts,
                                             const uint32_t *__restrict__ trow, uint32_t m,
                                             eg_mp_carry<typename Op::A> *__restrict__ carry, const Op &op,
                                             eg_red2 &redf, const G &gather, uint64_t pol) {
    constexpr uint32_t CH = 32u * U;  // entries per chunk
    using V = typename Op::V;
    using A = typename Op::A;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t E0 = t * (uint32_t)TILE_E;
    const uint32_t E1 = min(E0 + (uint32_t)TILE_E, m);
    uint32_t head_row, tile_next;
    uint32_t rbefore = 0;  // MK: row of the entry before the current chunk
    uint32_t sb_end = 0;   // MK: entry E1 begins a row
    if constexpr (MK) {
        const uint32_t first = __ldg(trow + E0 / EG_TROW_SPAN);
        const uint32_t sb0 = __ldg(starts + (E0 >> 5)) & 1u;  // E0 is a multiple of 32
        head_row = (E0 > 0 && !sb0) ? first : EG_MP_NONE;
        rbefore = first - sb0;  // wraps to 0xffffffff before entry 0: + 1 gives row 0
        sb_end = E1 < m ? __ldg(starts + (E1 >> 5)) & 1u : 0u;
        tile_next = EG_MP_NONE;  // (not used: rows are found from the bits)
    } else {
        const uint32_t first = __ldg(rid + E0);
        head_row = (E0 > 0 && __ldg(rid + E0 - 1) == first) ? first : EG_MP_NONE;
        tile_next = E1 < m ? __ldg(rid + E1) : EG_MP_NONE;
    }
    uint32_t crow = EG_MP_NONE;
    A cval = op.zero();
    bool head_done = false;
    A head_val = op.zero();
    auto finish = [&](uint32_t row, const A &val) {
        if (row == EG_MP_NONE) return;
        if (row == head_row) {
            head_done = true;
            head_val = val;
            return;
        }
        const float2 d = op.emit(row, val);
        if (REDUCE) redf.add(d);
    };
    // prefetched next chunk (PF >= 1): row ids (or MK: row-start word) and columns
    uint32_t rn[U], un[U], mwn = 0;
    uint32_t rg[U], mwg = 0;  // PF 2: rows (MK: row-start word) of the chunk whose gathers are in flight
    V vg[U];                  // PF 2: its gathered values
    auto load = [&](uint32_t cb, uint32_t (&rr)[U], uint32_t &mw, uint32_t (&uu)[U]) {
        if constexpr (MK) eg_coom_load<U, HINT>(col, starts, cb, E1, lane, mw, uu, pol);
        else eg_coov_load<U, HINT>(rid, col, cb, E1, lane, rr, uu, pol);
    };
    if (PF) load(E0, rn, mwn, un);
    if constexpr (PF == 2) {  // prologue: the first chunk's gathers, the second chunk's words
#pragma unroll
        for (int k = 0; k < U; k++) {
            const bool in = MK ? E0 + U * lane + k < E1 : rn[k] != EG_MP_NONE;
            if constexpr (!MK) rg[k] = rn[k];
            vg[k] = in ? gather(E0 + U * lane + k, un[k]) : V();
        }
        mwg = mwn;
        if (E0 + CH < E1) load(E0 + CH, rn, mwn, un);
    }
    for (uint32_t base = E0; base < E1; base += CH) {
        const uint32_t e = base + U * lane;
        uint32_t r[U], u[U], mw = 0;
        V v[U];
        if constexpr (PF == 2) {
            // this chunk's values arrived during the previous chunk's scan;
            // issue the next chunk's gathers and load the one after, then scan
#pragma unroll
            for (int k = 0; k < U; k++) {
                if constexpr (!MK) r[k] = rg[k];
                v[k] = vg[k];
            }
            mw = mwg;
            if (base + CH < E1) {
#pragma unroll
                for (int k = 0; k < U; k++) {
                    const bool in = MK ? e + CH + k < E1 : rn[k] != EG_MP_NONE;
                    if constexpr (!MK) rg[k] = rn[k];
                    vg[k] = in ? gather(e + CH + k, un[k]) : V();
                }
                mwg = mwn;
                if (base + 2 * CH < E1) load(base + 2 * CH, rn, mwn, un);
            }
            if constexpr (MK) eg_mask_rows<U>(mw, lane, base, E1, rbefore, r);
        } else {
            if (PF) {
#pragma unroll
                for (int k = 0; k < U; k++) {
                    if constexpr (!MK) r[k] = rn[k];
                    u[k] = un[k];
                }
                mw = mwn;
                if (base + CH < E1) load(base + CH, rn, mwn, un);
            } else {
                load(base, r, mw, u);
            }
            if constexpr (MK) {
                // gathers first: the row computation waits on nothing they need
#pragma unroll
                for (int k = 0; k < U; k++) v[k] = e + k < E1 ? gather(e + k, u[k]) : V();
                eg_mask_rows<U>(mw, lane, base, E1, rbefore, r);
            } else {
#pragma unroll
                for (int k = 0; k < U; k++) v[k] = r[k] != EG_MP_NONE ? gather(e + k, u[k]) : V();
            }
        }
        // row of the entry after this lane's last one
        uint32_t nxt = __shfl_down_sync(EG_FULL_MASK, r[0], 1);
        if (lane == 31) {
            if constexpr (MK) {
                if (base + CH < E1) nxt = r[U - 1] + (__ldg(starts + ((base + CH) >> 5)) & 1u);
                else nxt = E1 < m ? r[U - 1] + sb_end : EG_MP_NONE;
            } else {
                nxt = base + CH < E1 ? __ldg(rid + base + CH) : tile_next;
            }
        }
        const uint32_t prev_last = __shfl_up_sync(EG_FULL_MASK, r[U - 1], 1);
        // local runs: head run (from entry 0), middle runs, tail run (to entry U-1)
        A hsum = op.add(op.zero(), v[0]);
        A run = hsum;
        bool multi = false;
#pragma unroll
        for (int k = 1; k < U; k++) {
            if (r[k] != r[k - 1]) {
                if (!multi) hsum = run;  // the head run closed at k-1
                else finish(r[k - 1], run);
                multi = true;
                run = op.add(op.zero(), v[k]);
            } else {
                run = op.add(run, v[k]);
            }
        }
        if (!multi) hsum = run;
        // segmented scan of the tail runs across lanes
        A x = run;
        bool f = multi || lane == 0 || prev_last != r[0];
        if (lane == 0 && !multi && r[0] == crow) x = op.merge(cval, x);
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const A px = eg_shfl_up(x, off);
            const bool pf = __shfl_up_sync(EG_FULL_MASK, f, off);
            if (lane >= (uint32_t)off) {
                if (!f) x = op.merge(px, x);
                f = f || pf;
            }
        }
        // carry into this lane's head run (multi-run lanes)
        const A prevS = eg_shfl_up(x, 1);
        if (multi) {
            A tot = hsum;
            if (lane == 0) {
                if (r[0] == crow) tot = op.merge(cval, hsum);
            } else if (prev_last == r[0]) {
                tot = op.merge(prevS, hsum);
            }
            finish(r[0], tot);
        }
        if (nxt != r[U - 1]) finish(r[U - 1], x);
        crow = __shfl_sync(EG_FULL_MASK, r[U - 1], 31);
        cval = eg_shfl_idx(x, 31);
        rbefore = crow;  // MK: the next chunk starts after this row's entry
    }
    const uint32_t hmask = __ballot_sync(EG_FULL_MASK, head_done);
    if (lane == 0) {
        const bool tail_open = E1 < m && crow != EG_MP_NONE && (MK ? sb_end == 0u : tile_next == crow);
        carry[t].tail_row = tail_open ? crow : EG_MP_NONE;
        carry[t].tail_val = cval;
        carry[t].head_row = hmask ? head_row : EG_MP_NONE;
    }
    if (hmask) {
        const A hv = eg_shfl_idx(head_val, __ffs(hmask) - 1);
        if (lane == 0) carry[t].head_val = hv;
    }
}

// U entries per lane (U = 4 or 8): lane l of a warp holds entries
// base+U*l .. base+U*l+U-1 (128-bit loads of rid and col), sums the runs of
// equal rows among them locally, and one segmented scan per 32*U entries
// (flag form: a lane whose last run starts inside it, or whose row differs
// from the previous lane's last row, starts a segment) joins runs that cross
// lanes.  A run is emitted by the lane holding its last entry; the run open
// after lane 31 is carried to the next chunk.  Tiles are multiples of 32*U
// entries, so only the last tile has padding entries (row EG_MP_NONE, never
// emitted).
//
// PF 1: the next chunk's rid/col words are loaded before the current chunk's
// gathers, so the streaming loads of one chunk overlap the gathers and scan
// of the previous one.  PF 2: in addition the next chunk's gathers are issued
// before the current chunk's scan, so their latency hides behind the scan.  MINB: resident CTAs per SM asked of the compiler,
// which bounds the registers per thread (6: 42, 8: every warp slot, 32).
// HINT: cache hints on the streamed words (eg_stream_ld4).
// MK: rows from the row-start bits `starts` and the row samples `trow`
// (eg_mask_rows) instead of the row ids: 4.1 instead of 8 streamed bytes per
// entry, for layouts whose rows 0 .. last all have entries.
template <class Op, int TILE_E, int U, bool REDUCE, int PF = 0, int MINB = 6, int HINT = 0, bool MK = false>
__global__ void __launch_bounds__(256, MINB) k_coov_rows(const uint32_t *__restrict__ rid,
                                                         const uint32_t *__restrict__ col, uint32_t m, uint32_t ntiles,
                                                         eg_mp_carry<typename Op::A> *__restrict__ carry,
                                                         double2 *__restrict__ part, Op op,
                                                         const uint32_t *__restrict__ starts = nullptr,
                                                         const uint32_t *__restrict__ trow = nullptr) {
    static_assert(U == 4 || U == 8, "4 or 8 entries per lane");
    static_assert(TILE_E % (32 * U) == 0, "tiles hold whole chunks");
    static_assert(!MK || TILE_E % EG_TROW_SPAN == 0, "tiles start at a row sample");
    __shared__ double2 s_red[8];
    if (!op.active()) return;
    op.setup();
    const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t pol = HINT ? eg_l2_evict_first_policy() : 0;
    eg_red2 redf;
    if (t < ntiles)
        eg_coov_tile<Op, TILE_E, U, REDUCE, PF, HINT, MK>(
            t, rid, col, starts, trow, m, carry, op, redf, [&](uint32_t e, uint32_t u) { return op.gather(e, u); },
            pol);
    if (REDUCE) eg_coov_reduce(redf, s_red, 8, part);
}
