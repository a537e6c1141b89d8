// Builds PageRank's destination-partition layout (eg_pcols) from the
// relabelled CSC, on the device, once per graph and partition size.
//
// The relabelled CSC lists each row's entries by ascending source.  Two
// stable radix sorts put the entries in (partition of the row, source, row)
// order: by source first, then by partition.  Each partition's entries are
// then written at the next chunk boundary as 2-byte rows within the
// partition, with a bit per entry marking where a run (the entries of one
// source) begins; a chunk always begins a run, so a warp can take any chunk
// without looking at the one before.  The runs' sources are the words the
// kernel gathers through.  Segments of at most 256 .. 2048 chunks (by the
// size of the graph) split the long partitions, and are listed longest first
// for the kernel's queue.
#include <algorithm>
#include <vector>

#include "eg_internal.cuh"

#ifndef EG_PC_SEG_MIN
#define EG_PC_SEG_MIN 256    // chunks per segment at most: 64K entries ..
#endif
#ifndef EG_PC_SEG_MAX
#define EG_PC_SEG_MAX 2048   // .. 512K entries
#endif
#ifndef EG_PC_SEG_PER_SM
#define EG_PC_SEG_PER_SM 4   // segments per SM the size aims at (RMAT-24 row pass: 2 or 4 0.484 ms, 8 0.516)
#endif

namespace {
__global__ void k_pc_keys(const uint32_t *__restrict__ rowid, uint64_t M, uint32_t shift, uint32_t *keys,
                          uint32_t *idx) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < M; e += (uint64_t)gridDim.x * blockDim.x) {
        keys[e] = rowid[e] >> shift;
        idx[e] = (uint32_t)e;
    }
}

// First entry of every partition in the sorted order: the CSC row pointer
// of the partition's first row (rows are grouped by partition in row order).
__global__ void k_pc_bounds(const uint32_t *__restrict__ ptr, uint32_t rows, uint32_t parts, uint32_t shift,
                            uint32_t *out) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p <= parts; p += gridDim.x * blockDim.x) {
        const uint64_t r = (uint64_t)p << shift;
        out[p] = ptr[r < rows ? r : rows];
    }
}

// One thread per padded position o: its row within the partition (2^shift
// for padding), its run-start bit (a ballot per 32 positions) and its source.
// EG_PC_CHUNK is 256: 8 entries per lane of a warp.
__global__ void k_pc_fill(const uint32_t *__restrict__ cbase, const uint32_t *__restrict__ ebase, uint32_t parts,
                          uint32_t shift, const uint32_t *__restrict__ order, const uint32_t *__restrict__ src,
                          const uint32_t *__restrict__ row, uint64_t npos, uint16_t *__restrict__ out_row,
                          uint32_t *__restrict__ flags, uint32_t *__restrict__ spos) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;  // a multiple of 32: warps stay whole
    for (uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; o < npos; o += stride) {
        const uint64_t c = o / EG_PC_CHUNK;
        uint32_t lo = 0, hi = parts;  // cbase[lo] <= c < cbase[hi]
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if ((uint64_t)cbase[mid] <= c) lo = mid;
            else hi = mid;
        }
        const uint64_t j = o - (uint64_t)cbase[lo] * EG_PC_CHUNK;
        const uint64_t cnt = (uint64_t)ebase[lo + 1] - ebase[lo];
        bool start = false;
        uint32_t r = 1u << shift, s = 0;
        if (j < cnt) {
            const uint64_t i = ebase[lo] + j;
            const uint32_t x = order[i];
            s = src[x];
            r = row[x] & ((1u << shift) - 1u);
            start = j == 0 || (o % EG_PC_CHUNK) == 0 || src[order[i - 1]] != s;
        }
        // chunks are stored transposed: lane l's 16 bytes hold the rows of
        // entries l, l + 32, ..., l + 224
        out_row[(o & ~(uint64_t)(EG_PC_CHUNK - 1)) | ((o & 31) << 3) | ((o >> 5) & 7)] = (uint16_t)r;
        spos[o] = s;
        const uint32_t b = __ballot_sync(EG_FULL_MASK, start);
        if ((threadIdx.x & 31) == 0) flags[o >> 5] = b;
    }
}

// Each entry's run within its chunk (the run starts at or before it, less
// one), stored transposed like the rows: lane l's 8 bytes hold entries l,
// l + 32, ..., l + 224.
__global__ void k_pc_ridx(const uint32_t *__restrict__ flags, uint64_t npos, uint8_t *__restrict__ ridx) {
    for (uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; o < npos; o += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t c = o / EG_PC_CHUNK;
        const uint32_t e = (uint32_t)(o % EG_PC_CHUNK), j = e >> 5, b = e & 31u;
        const uint32_t *fw = flags + c * (EG_PC_CHUNK / 32);
        uint32_t q = __popc(fw[j] & (0xffffffffu >> (31u - b)));
        for (uint32_t i = 0; i < j; i++) q += __popc(fw[i]);
        ridx[c * EG_PC_CHUNK + b * 8u + j] = (uint8_t)(q - 1u);
    }
}

__global__ void k_pc_popc(const uint32_t *__restrict__ flags, uint64_t nwords, uint32_t *cnt) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords; w += (uint64_t)gridDim.x * blockDim.x)
        cnt[w] = __popc(flags[w]);
}

// The source of every run, and the run of every chunk's first entry.
__global__ void k_pc_runs(const uint32_t *__restrict__ flags, const uint32_t *__restrict__ wbase,
                          const uint32_t *__restrict__ spos, uint64_t npos, uint32_t *__restrict__ rsrc,
                          uint32_t *__restrict__ crun) {
    for (uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; o < npos; o += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t f = flags[o >> 5], b = (uint32_t)(o & 31);
        if (!((f >> b) & 1u)) continue;
        const uint32_t r = wbase[o >> 5] + __popc(f & ((1u << b) - 1u));
        rsrc[r] = spos[o];
        if (o % EG_PC_CHUNK == 0) crun[o / EG_PC_CHUNK] = r;
    }
}

uint32_t pc_grid(eg_ctx *ctx, uint64_t work) {
    uint64_t b = (work + 255) / 256;
    const uint64_t cap = (uint64_t)ctx->sm_count * 16;
    return (uint32_t)(b > cap ? cap : (b ? b : 1));
}
}  // namespace

int eg_build_pcols(eg_graph *g, uint32_t shift) {
    eg_pcols &pc = g->pcol;
    if (pc.shift == shift && g->relabeled) return EG_OK;
    if (!g->relabeled) return eg_fail(EG_ENOTBUILT, "partition layout needs the relabelled CSC");
    if (shift < 8 || shift > 15) return eg_fail(EG_EINVAL, "partitions of 2^%u rows (2^8 .. 2^15)", shift);
    eg_ctx *ctx = g->ctx;
    const uint64_t M = g->m;
    const uint32_t rows = g->csc_p_rows;
    if (M >= (1ull << 32) - EG_PC_CHUNK * 65536ull)
        return eg_fail(EG_EINVAL, "partition layout: %llu entries, fewer than 2^32 needed", (unsigned long long)M);
    pc.shift = 0;
    const uint32_t P = rows ? ((rows - 1) >> shift) + 1 : 0;
    eg_buf ka, va, kb, vb, kc, vc, bnd, sp, wcnt, wbase, fl;  // fl: the run-start bits (build only)
    int rc = EG_OK;
    auto cleanup = [&]() {
        cudaStreamSynchronize(ctx->stream);
        for (eg_buf *b : {&ka, &va, &kb, &vb, &kc, &vc, &bnd, &sp, &wcnt, &wbase, &fl}) eg_buf_free(ctx, *b);
    };
#define PTRY(x)            \
    do {                   \
        rc = (x);          \
        if (rc != EG_OK) { \
            cleanup();     \
            return rc;     \
        }                  \
    } while (0)
    // partition bounds in entries, then each partition padded to whole chunks
    PTRY(eg_buf_ensure(ctx, bnd, ((uint64_t)P + 1) * 8 + 16));
    uint32_t *ebase = bp<uint32_t>(bnd), *cbase_d = ebase + P + 1;
    k_pc_bounds<<<pc_grid(ctx, P + 1), 256, 0, ctx->stream>>>(bp<uint32_t>(g->csc_p.ptr), rows, P, shift, ebase);
    ctx->launches++;
    std::vector<uint32_t> eb(P + 1), cb(P + 1);
    if (cudaMemcpyAsync(eb.data(), ebase, ((uint64_t)P + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        PTRY(eg_fail(EG_ECUDA, "partition bounds: %s", cudaGetErrorString(cudaGetLastError())));
    uint64_t chunks = 0;
    for (uint32_t p = 0; p < P; p++) {
        cb[p] = (uint32_t)chunks;
        chunks += ((uint64_t)eb[p + 1] - eb[p] + EG_PC_CHUNK - 1) / EG_PC_CHUNK;
    }
    // segments: about four per SM of the whole work, so that the longest-
    // first queue balances the SMs, but as long as that allows, since every
    // segment zeroes and writes out a partition's row sums
    uint64_t segc = EG_PC_SEG_MIN;
    while (segc < EG_PC_SEG_MAX && segc * EG_PC_SEG_PER_SM * (uint64_t)ctx->sm_count < chunks) segc *= 2;
    std::vector<uint4> segs;
    for (uint32_t p = 0; p < P; p++) {
        const uint64_t c0 = cb[p], nch = (p + 1 < P ? cb[p + 1] : chunks) - c0;
        const uint64_t ns = nch ? (nch + segc - 1) / segc : 1;
        for (uint64_t s = 0; s < ns; s++)
            segs.push_back(make_uint4((uint32_t)(c0 + s * nch / ns), (uint32_t)(c0 + (s + 1) * nch / ns), p,
                                      (uint32_t)ns));
    }
    cb[P] = (uint32_t)chunks;
    std::stable_sort(segs.begin(), segs.end(), [](const uint4 &a, const uint4 &b) { return a.y - a.x > b.y - b.x; });
    const uint64_t npos = chunks * EG_PC_CHUNK;
    if (cudaMemcpyAsync(cbase_d, cb.data(), ((uint64_t)P + 1) * 4, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
        PTRY(eg_fail(EG_ECUDA, "partition chunk offsets"));
    // (source, row) order, then stably by partition: positions into that order
    const uint64_t len = M + 1;
    for (eg_buf *b : {&ka, &va, &kb, &vb, &kc, &vc}) PTRY(eg_buf_ensure(ctx, *b, len * 4));
    uint32_t *ks = bp<uint32_t>(ka), *vs = bp<uint32_t>(va);
    if (M) {
        if (cudaMemcpyAsync(ka.p, g->csc_p.col.p, M * 4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess ||
            cudaMemcpyAsync(va.p, g->csc_p.rid.p, M * 4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
            PTRY(eg_fail(EG_ECUDA, "partition layout copy"));
        const int bits = g->n <= 1 ? 1 : 32 - __builtin_clz(g->n - 1);
        PTRY(eg_radix_sort(ctx, bp<uint32_t>(ka), bp<uint32_t>(va), bp<uint32_t>(kb), bp<uint32_t>(vb), M, bits, &ks,
                           &vs));
    }
    // ks: sources ascending, vs: their rows; then the partition keys into the
    // other pair, sorted with (kc, vc) as the temporary pair
    eg_buf &fk = ks == bp<uint32_t>(ka) ? kb : ka;
    eg_buf &fv = vs == bp<uint32_t>(va) ? vb : va;
    uint32_t *ord = bp<uint32_t>(fv);
    if (M) {
        k_pc_keys<<<pc_grid(ctx, M), 256, 0, ctx->stream>>>(vs, M, shift, bp<uint32_t>(fk), bp<uint32_t>(fv));
        ctx->launches++;
        uint32_t *ko = nullptr;
        const int pbits = P <= 1 ? 1 : 32 - __builtin_clz(P - 1);
        PTRY(eg_radix_sort(ctx, bp<uint32_t>(fk), bp<uint32_t>(fv), bp<uint32_t>(kc), bp<uint32_t>(vc), M, pbits, &ko,
                           &ord));
    }
    // keep ks, vs and ord; the sources per padded position go to a new buffer
    cudaStreamSynchronize(ctx->stream);
    for (eg_buf *b : {&ka, &va, &kb, &vb, &kc, &vc})
        if (b->p != ks && b->p != vs && b->p != ord) eg_buf_free(ctx, *b);
    PTRY(eg_buf_ensure(ctx, sp, npos * 4 + 16));
    uint32_t *spos = bp<uint32_t>(sp);
    PTRY(eg_buf_ensure(ctx, pc.dst, npos * 2 + 16));
    PTRY(eg_buf_ensure(ctx, fl, (npos / 32) * 4 + 16));
    PTRY(eg_buf_ensure(ctx, pc.crun, chunks * 4 + 16));
    PTRY(eg_buf_ensure(ctx, pc.ridx, npos + 16));
    if (npos) {
        k_pc_fill<<<pc_grid(ctx, npos), 256, 0, ctx->stream>>>(cbase_d, ebase, P, shift, ord, ks, vs, npos,
                                                              bp<uint16_t>(pc.dst), bp<uint32_t>(fl), spos);
        ctx->launches++;
        k_pc_ridx<<<pc_grid(ctx, npos), 256, 0, ctx->stream>>>(bp<uint32_t>(fl), npos, bp<uint8_t>(pc.ridx));
        ctx->launches++;
    }
    // run numbers: an exclusive scan of the flag words' bit counts
    const uint64_t nwords = npos / 32;
    PTRY(eg_buf_ensure(ctx, wcnt, nwords * 4 + 16));
    rc = eg_buf_ensure(ctx, wbase, (nwords + 1) * 4 + 16);
    uint32_t runs = 0;
    if (rc == EG_OK && nwords) {
        k_pc_popc<<<pc_grid(ctx, nwords), 256, 0, ctx->stream>>>(bp<uint32_t>(fl), nwords, bp<uint32_t>(wcnt));
        ctx->launches++;
        rc = eg_exscan_u32(ctx, bp<uint32_t>(wcnt), bp<uint32_t>(wbase), nwords);
        if (rc == EG_OK &&
            (cudaMemcpyAsync(&runs, bp<uint32_t>(wbase) + nwords, 4, cudaMemcpyDeviceToHost, ctx->stream) !=
                 cudaSuccess ||
             cudaStreamSynchronize(ctx->stream) != cudaSuccess))
            rc = eg_fail(EG_ECUDA, "partition runs: %s", cudaGetErrorString(cudaGetLastError()));
        if (rc == EG_OK) rc = eg_buf_ensure(ctx, pc.rsrc, (uint64_t)runs * 4 + 16);
        if (rc == EG_OK) {
            k_pc_runs<<<pc_grid(ctx, npos), 256, 0, ctx->stream>>>(bp<uint32_t>(fl), bp<uint32_t>(wbase), spos,
                                                                  npos, bp<uint32_t>(pc.rsrc), bp<uint32_t>(pc.crun));
            ctx->launches++;
        }
    }
    if (rc != EG_OK) {
        cleanup();
        return rc;
    }
    // segments, accumulators, tickets
    PTRY(eg_buf_ensure(ctx, pc.seg, segs.size() * sizeof(uint4) + 16));
    PTRY(eg_buf_ensure(ctx, pc.acc, (uint64_t)rows * 8 + 16));
    PTRY(eg_buf_ensure(ctx, pc.ticket, ((uint64_t)P + 2) * 4 + 16));
    if ((!segs.empty() && cudaMemcpyAsync(pc.seg.p, segs.data(), segs.size() * sizeof(uint4), cudaMemcpyHostToDevice,
                                          ctx->stream) != cudaSuccess) ||
        cudaMemsetAsync(pc.acc.p, 0, (uint64_t)rows * 8 + 16, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(pc.ticket.p, 0, ((uint64_t)P + 2) * 4 + 16, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        PTRY(eg_fail(EG_ECUDA, "partition layout: %s", cudaGetErrorString(cudaGetLastError())));
#undef PTRY
    cleanup();
    pc.parts = P;
    pc.segs = (uint32_t)segs.size();
    pc.chunks = chunks;
    pc.runs = runs;
    pc.shift = shift;
    return EG_OK;
}
