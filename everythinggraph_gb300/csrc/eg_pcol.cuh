// Row sums over the destination-partition layout (eg_pcols, built by
// eg_pcol.cu): PageRank's pull iteration with the contribution of each
// source gathered once per partition instead of once per entry.
//
// The row kernel (eg_mp.cuh) walks the CSC in row order, so consecutive
// entries name unrelated sources and nearly every entry gathers its own
// 32-byte sector (0.98 sectors per entry on directed RMAT-24 before L1).
// Here a partition's entries are ordered by source: all entries of source
// u into the partition form one run, whose contribution is loaded once and
// added into the rows of the run's entries, and consecutive runs are
// ascending sources, so the loads of a warp share sectors (0.19 sectors per
// entry for partitions of 8K rows on directed RMAT-24).  The streamed words are 3 bytes per
// entry (the row within the partition, and the entry's run within its
// 256-entry chunk), and 4 bytes per run (its source).
//
// A CTA owns one segment of a partition's chunks at a time (persistent CTAs
// take segments from a queue, longest first) and sums into the partition's
// rows held in shared memory.  Sums are kept as unsigned 64-bit fixed point
// (a power-of-two unit chosen by the host so that no sum reaches 2^61 units;
// a contribution c becomes round(c / unit), an error of at most half a unit
// per term): integer adds give the same bits in any order, so
// the result does not depend on which warp or CTA added first.  A partition covered by one
// segment is finished from shared memory; the segments of a longer partition
// add their sums into a global accumulator, and the last to finish (a ticket
// per partition) finishes the rows and clears the accumulator.
#pragma once
#include "eg_mp.cuh"

#ifndef EG_PC_THREADS
#define EG_PC_THREADS 1024  // (512 with two CTAs per SM: 0.553 against 0.505 ms on RMAT-24)
#endif
#define EG_PC_CTAS (1024 / EG_PC_THREADS)  // resident CTAs per SM (64 registers a thread)
#define EG_PC_WARPS (EG_PC_THREADS / 32)

// Shared memory of k_pcol_rows with partitions of 2^SHIFT rows: the row
// sums as 64-bit fixed point (one slot more for the padding entries), the
// low 32-bit words of every row, then the high words, and each warp's run
// values (64-bit) for the chunk in hand.  A term is added to the low word
// with a 32-bit integer atomic; when that add wraps, the high word gets one
// more with the term's high half: every sum is exact, so its bits do not
// depend on the order of the adds (and 32-bit integer adds are the shared
// memory atomics that the hardware carries out natively).
template <int SHIFT>
struct eg_pc_smem {
    static constexpr size_t word_bytes = (((size_t)(1u << SHIFT) + 1) * 4 + 15) & ~(size_t)15;
    static constexpr size_t acc_bytes = 2 * word_bytes;
    static constexpr size_t bytes = acc_bytes + (size_t)EG_PC_WARPS * EG_PC_CHUNK * 8;
};

// round(x) for 0 <= x < 2^64 as an unsigned 64-bit integer, from 32-bit
// conversions only (a 64-bit float-to-integer conversion runs on the FP64
// pipe, which is narrow on this GPU).  hi = floor(x / 2^32) and
// x - hi * 2^32 (exact: both are multiples of x's ulp) are floats; the low
// part has a fraction only when x < 2^24, where hi = 0, so rounding it to
// the nearest integer rounds x.
__device__ __forceinline__ unsigned long long eg_f2u64_rn(float x) {
    const float hf = truncf(x * 2.3283064365386963e-10f);  // x / 2^32
    const float lf = fmaf(-hf, 4294967296.0f, x);           // x - hi * 2^32
    return ((unsigned long long)__float2uint_rz(hf) << 32) | __float2uint_rn(lf);
}

// The unsigned 64-bit value hi * 2^32 + lo rounded to the nearest float
// (ties to even), from 32-bit integer operations for the same reason.
__device__ __forceinline__ float eg_u642f_rn(uint32_t hi, uint32_t lo) {
    if (hi == 0u) return __uint2float_rn(lo);
    const int lz = __clz(hi);
    const int sh = 40 - lz;  // bits below the 24-bit significand (9 .. 40)
    const unsigned long long v = ((unsigned long long)hi << 32) | lo;
    uint32_t mant = (uint32_t)(v >> sh);
    const unsigned long long rem = v & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    int e = 63 - lz;  // exponent of the leading bit
    if (rem > half || (rem == half && (mant & 1u))) mant++;
    if (mant == (1u << 24)) {
        mant >>= 1;
        e++;
    }
    return __uint_as_float(((uint32_t)(e + 127) << 23) | (mant & 0x7fffffu));
}

// One streamed 4-byte word (read once per pass): not kept in L1, first in
// line for L2 eviction.
__device__ __forceinline__ uint32_t eg_stream_ldu(const uint32_t *p, uint64_t pol) {
    uint32_t v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}

// A warp's chunk: the rows of entries lane, lane + 32, ..., lane + 224 (one
// 16-byte word per lane: the layout stores each chunk transposed), the runs
// (within the chunk) of the same entries (8 bytes per lane, byte j: entry
// lane + 32j), the chunk's first run.
struct eg_pc_chunk {
    uint4 d8;
    uint2 ri;
    uint32_t rb;
};
__device__ __forceinline__ uint2 eg_stream_ld2(const uint32_t *p, uint64_t pol) {
    uint2 v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
        : "=r"(v.x), "=r"(v.y)
        : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void eg_pc_load(const uint32_t *__restrict__ dst, const uint32_t *__restrict__ ridx,
                                           const uint32_t *__restrict__ crun, uint64_t c, uint32_t lane,
                                           uint64_t pol, eg_pc_chunk &k) {
    k.d8 = eg_stream_ld4<1>(dst + c * (EG_PC_CHUNK / 2) + 4 * lane, pol);
    k.ri = eg_stream_ld2(ridx + c * (EG_PC_CHUNK / 4) + 2 * lane, pol);
    k.rb = __ldg(crun + c);
}

// The chunk's run count (the run of its last entry, lane 31's byte 7, plus
// one: padding entries continue the last run) and, when it has at most 64
// runs, the sources of runs lane and lane + 32.
__device__ __forceinline__ uint32_t eg_pc_sources(const eg_pc_chunk &k, const uint32_t *__restrict__ rsrc,
                                                  uint32_t lane, uint32_t &u1, uint32_t &u2) {
    const uint32_t nr = __shfl_sync(EG_FULL_MASK, k.ri.y >> 24, 31) + 1u;
    u1 = u2 = 0u;
    if (nr <= 64) {
        if (lane < nr) u1 = __ldg(rsrc + k.rb + lane);
        if (lane + 32 < nr) u2 = __ldg(rsrc + k.rb + lane + 32);
    }
    return nr;
}

template <class Op, int SHIFT, bool REDUCE>
__global__ void __launch_bounds__(EG_PC_THREADS, EG_PC_CTAS)
    k_pcol_rows(const uint4 *__restrict__ seg, uint32_t nseg, const uint32_t *__restrict__ dst,
                const uint32_t *__restrict__ ridx, const uint32_t *__restrict__ crun,
                const uint32_t *__restrict__ rsrc, unsigned long long *__restrict__ gacc,
                uint32_t *__restrict__ ticket, uint32_t parts, uint32_t rows, double2 *__restrict__ part, Op op,
                float fx, float fx_inv) {
    using T = unsigned long long;
    constexpr uint32_t D = 1u << SHIFT;
    extern __shared__ __align__(16) unsigned char eg_pc_sm[];
    using SM = eg_pc_smem<SHIFT>;
    uint32_t *slo = reinterpret_cast<uint32_t *>(eg_pc_sm);                    // low words
    uint32_t *shi = reinterpret_cast<uint32_t *>(eg_pc_sm + SM::word_bytes);  // high words
    auto row_sum = [&](uint32_t l) -> float { return eg_u642f_rn(shi[l], slo[l]) * fx_inv; };
    __shared__ double2 s_red[32];
    __shared__ uint32_t s_seg;
    __shared__ int s_last;
    if (!op.active()) return;
    op.setup();
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    T *wv = reinterpret_cast<T *>(eg_pc_sm + SM::acc_bytes) + warp * EG_PC_CHUNK;
    const uint64_t pol = eg_l2_evict_first_policy();
    eg_red2 redf;
    for (;;) {
        if (tid == 0) s_seg = atomicAdd(ticket + parts, 1u);
        __syncthreads();
        const uint32_t si = s_seg;
        if (si >= nseg) break;
        const uint4 sg = seg[si];
        const uint32_t c1 = sg.y, p = sg.z, nsp = sg.w;
        for (uint32_t i = tid; i <= D; i += EG_PC_THREADS) {
            slo[i] = 0u;
            shi[i] = 0u;
        }
        __syncthreads();
        // a two-stage pipeline per warp: while chunk c is summed, the words
        // of chunk c + 2W are in flight and the run sources of chunk c + W
        // are loaded, so that c's gathers wait for one memory round trip
        uint64_t c = (uint64_t)sg.x + warp, cn = c + EG_PC_WARPS;
        eg_pc_chunk k = {}, kn = {};
        uint32_t nr = 0, u1 = 0, u2 = 0;
        if (c < c1) {
            eg_pc_load(dst, ridx, crun, c, lane, pol, k);
            nr = eg_pc_sources(k, rsrc, lane, u1, u2);
        }
        if (cn < c1) eg_pc_load(dst, ridx, crun, cn, lane, pol, kn);
        while (c < c1) {
            const uint64_t cnn = cn + EG_PC_WARPS;
            eg_pc_chunk knn = kn;
            if (cnn < c1) eg_pc_load(dst, ridx, crun, cnn, lane, pol, knn);
            uint32_t nrn = 0, un1 = 0, un2 = 0;
            if (cn < c1) nrn = eg_pc_sources(kn, rsrc, lane, un1, un2);
            // one contribution per run (consecutive runs: ascending sources);
            // a chunk with more than 64 runs loads all of the lane's source
            // words, then all its gathers
            if (nr <= 64) {
                const uint32_t i2 = lane + 32;
                const float v1 = lane < nr ? op.gather(0u, u1) : 0.f;
                const float v2 = i2 < nr ? op.gather(0u, u2) : 0.f;
                if (lane < nr) wv[lane] = eg_f2u64_rn(v1 * fx);
                if (i2 < nr) wv[i2] = eg_f2u64_rn(v2 * fx);
            } else {
                uint32_t us[EG_PC_CHUNK / 32];
                float vs[EG_PC_CHUNK / 32];
#pragma unroll
                for (int i = 0; i < EG_PC_CHUNK / 32; i++) {
                    const uint32_t r = lane + 32u * i;
                    us[i] = r < nr ? __ldg(rsrc + k.rb + r) : 0u;
                }
#pragma unroll
                for (int i = 0; i < EG_PC_CHUNK / 32; i++) {
                    const uint32_t r = lane + 32u * i;
                    vs[i] = r < nr ? op.gather(0u, us[i]) : 0.f;
                }
#pragma unroll
                for (int i = 0; i < EG_PC_CHUNK / 32; i++) {
                    const uint32_t r = lane + 32u * i;
                    if (r < nr) wv[r] = eg_f2u64_rn(vs[i] * fx);
                }
            }
            __syncwarp();
            // entry 32j + lane: its row (16 bits) and its run (byte j)
            const uint32_t h[4] = {k.d8.x, k.d8.y, k.d8.z, k.d8.w};
#pragma unroll
            for (int j0 = 0; j0 < 8; j0 += 4) {
                uint32_t rw[4], old[4];
                T val[4];
#pragma unroll
                for (int jj = 0; jj < 4; jj++) {
                    const int j = j0 + jj;
                    const uint32_t q = ((j < 4 ? k.ri.x : k.ri.y) >> (8 * (j & 3))) & 0xffu;
                    rw[jj] = (j & 1) ? (h[j >> 1] >> 16) : (h[j >> 1] & 0xffffu);
                    val[jj] = wv[q];
                    old[jj] = atomicAdd(slo + rw[jj], (uint32_t)val[jj]);
                }
#pragma unroll
                for (int jj = 0; jj < 4; jj++) {
                    const uint32_t lo = (uint32_t)val[jj];
                    const uint32_t hv = (uint32_t)(val[jj] >> 32) + (old[jj] + lo < old[jj] ? 1u : 0u);
                    if (hv) atomicAdd(shi + rw[jj], hv);
                }
            }
            __syncwarp();
            c = cn;
            cn = cnn;
            k = kn;
            kn = knn;
            nr = nrn;
            u1 = un1;
            u2 = un2;
        }
        __syncthreads();
        const uint32_t row0 = p << SHIFT;
        const uint32_t nrows = rows - row0 < D ? rows - row0 : D;
        if (nsp == 1) {
            for (uint32_t l = tid; l < nrows; l += EG_PC_THREADS) {
                const float2 d = op.emit(row0 + l, row_sum(l));
                if (REDUCE) redf.add(d);
            }
        } else {
            for (uint32_t l = tid; l < nrows; l += EG_PC_THREADS) {
                const T a = ((T)shi[l] << 32) | (T)slo[l];
                if (a) atomicAdd(gacc + row0 + l, a);
            }
            __threadfence();
            __syncthreads();
            if (tid == 0) s_last = atomicAdd(ticket + p, 1u) == nsp - 1;
            __syncthreads();
            if (s_last) {
                __threadfence();
                for (uint32_t l = tid; l < nrows; l += EG_PC_THREADS) {
                    const T a = __ldcg(gacc + row0 + l);
                    gacc[row0 + l] = 0ull;
                    const float2 d = op.emit(row0 + l, eg_u642f_rn((uint32_t)(a >> 32), (uint32_t)a) * fx_inv);
                    if (REDUCE) redf.add(d);
                }
                if (tid == 0) ticket[p] = 0u;
            }
        }
        __syncthreads();  // s_seg and the shared sums are reused by the next segment
    }
    // the last CTA to leave resets the segment queue for the next launch
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(ticket + parts + 1, 1u) == gridDim.x - 1) {
            ticket[parts] = 0u;
            ticket[parts + 1] = 0u;
        }
    }
    eg_block_part<REDUCE>(redf, part, s_red);
}
