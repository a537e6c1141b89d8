// Context, device memory, graph input and the device layout builders
// (degree histogram, scan, stable radix sort, CSR/CSC and 2-D grid).
//
// The builders replace the reference loader (init_all.c): preload_graph
// (init_all.c:81-110), init_adj_sort (init_all.c:629-790) with its Ligra
// radix sort (radixSort_ligra.h:290-358) and offset back-fill
// (utils_ligra.h:212-214), and init_grid_sort (init_all.c:252-361).
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <time.h>

#include "eg_internal.cuh"

// ============================================================== errors
static thread_local char g_err[1024];

int eg_fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}
void eg_clear_error() { g_err[0] = 0; }

extern "C" const char *eg_last_error(void) { return g_err; }
extern "C" const char *eg_version(void) { return "everythinggraph_gb300 0.1 (sm_103a)"; }

// ============================================================== context
extern "C" int eg_open(int device, uint64_t hbm_budget_bytes, eg_ctx **out) {
    if (!out) return eg_fail(EG_EINVAL, "eg_open: out is NULL");
    *out = nullptr;
    int ndev = 0;
    EG_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return eg_fail(EG_EINVAL, "eg_open: device %d of %d", device, ndev);
    EG_CUDA(cudaSetDevice(device));
    eg_ctx *c = new eg_ctx();
    c->device = device;
    c->budget = hbm_budget_bytes;
    EG_CUDA(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device));
    EG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    EG_CUDA(cudaMallocHost(&c->h_pinned, 1 << 20));
    EG_CUDA(cudaHostGetDevicePointer(&c->h_pinned_dev, c->h_pinned, 0));
    *reinterpret_cast<uint32_t *>(static_cast<char *>(c->h_pinned) + EG_RB_FLAG_OFF) = 0;  // no readback yet
    EG_CUDA(cudaEventCreate(&c->ev0));
    EG_CUDA(cudaEventCreate(&c->ev1));
    for (cudaEvent_t &e : c->evk) EG_CUDA(cudaEventCreate(&e));
    EG_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (cudaEvent_t &e : c->ev_out) EG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    *out = c;
    return EG_OK;
}

namespace {
// One warp copies `words` to pinned host memory (and clears them); with a
// flag, lane 0 releases `seq` to the flag word after every lane's stores:
// the warp barrier orders the other lanes' stores before lane 0's
// system-scope fence (cumulativity), and the fence orders them before the
// flag store that the host reads with acquire semantics.
__global__ void k_readback(uint32_t *src, uint32_t *dst, uint32_t words, int clear, uint32_t *flag, uint32_t seq) {
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) {
        dst[i] = src[i];
        if (clear) src[i] = 0u;
    }
    if (flag) {
        __syncwarp();
        if (threadIdx.x == 0) {
            __threadfence_system();
            *(volatile uint32_t *)flag = seq;
        }
    }
}
__global__ void k_zero(uint32_t *p, uint64_t words) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < words; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = 0u;
}
}  // namespace

int eg_zero(eg_ctx *c, void *dev, uint64_t bytes, cudaStream_t st) {
    if ((bytes & 3) || ((uintptr_t)dev & 3)) return eg_fail(EG_EINVAL, "eg_zero: unaligned");
    const uint64_t words = bytes / 4;
    if (!words) return EG_OK;
    uint64_t blocks = (words + 255) / 256;
    if (blocks > (uint64_t)c->sm_count * 8) blocks = (uint64_t)c->sm_count * 8;
    k_zero<<<(uint32_t)blocks, 256, 0, st>>>(static_cast<uint32_t *>(dev), words);
    EG_LAUNCHED(c);
    return EG_OK;
}

static int readback_launch(eg_ctx *c, void *host_dst, const void *dev_src, uint32_t bytes, cudaStream_t st, bool clear,
                           uint32_t *flag_dev, uint32_t seq) {
    const uintptr_t off = (uintptr_t)host_dst - (uintptr_t)c->h_pinned;
    if ((uintptr_t)host_dst < (uintptr_t)c->h_pinned || off + bytes > EG_RB_FLAG_OFF || (off & 3) ||
        ((uintptr_t)dev_src & 3))
        return eg_fail(EG_EINVAL, "readback outside the pinned staging area");
    k_readback<<<1, 32, 0, st>>>(static_cast<uint32_t *>(const_cast<void *>(dev_src)),
                                 reinterpret_cast<uint32_t *>(static_cast<char *>(c->h_pinned_dev) + off),
                                 (bytes + 3) / 4, clear ? 1 : 0, flag_dev, seq);
    EG_LAUNCHED(c);
    return EG_OK;
}

int eg_readback(eg_ctx *c, void *host_dst, const void *dev_src, uint32_t bytes, cudaStream_t st, bool clear) {
    return readback_launch(c, host_dst, dev_src, bytes, st, clear, nullptr, 0);
}

int eg_readback_wait(eg_ctx *c, void *host_dst, const void *dev_src, uint32_t bytes, cudaStream_t st, bool clear) {
    uint32_t seq = ++c->rb_seq;
    if (seq == 0) seq = ++c->rb_seq;  // 0 is the flag's value before any readback
    uint32_t *flag_dev = reinterpret_cast<uint32_t *>(static_cast<char *>(c->h_pinned_dev) + EG_RB_FLAG_OFF);
    uint32_t *flag = reinterpret_cast<uint32_t *>(static_cast<char *>(c->h_pinned) + EG_RB_FLAG_OFF);
    // the flag holds an earlier value; make sure of it before the launch
    __atomic_store_n(flag, seq - 1u, __ATOMIC_SEQ_CST);
    __atomic_thread_fence(__ATOMIC_SEQ_CST);
    EG_TRY(readback_launch(c, host_dst, dev_src, bytes, st, clear, flag_dev, seq));
    timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (uint32_t i = 1;; i++) {
        if (__atomic_load_n(flag, __ATOMIC_ACQUIRE) == seq) return EG_OK;  // the words before it are visible
        if ((i & 4095u) == 0) {
            clock_gettime(CLOCK_MONOTONIC, &t1);
            if ((t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec) > 1.0) break;
        }
    }
    EG_CUDA(cudaStreamSynchronize(st));  // a device error surfaces here
    if (__atomic_load_n(flag, __ATOMIC_ACQUIRE) != seq) return eg_fail(EG_ETIMEOUT, "readback flag not raised");
    return EG_OK;
}

extern "C" int eg_host_alloc(uint64_t bytes, void **out) {
    if (!out) return eg_fail(EG_EINVAL, "NULL argument");
    *out = nullptr;
    if (bytes == 0) return EG_OK;
    const cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return eg_fail(EG_ENOMEM, "cudaHostAlloc(%llu): %s", (unsigned long long)bytes, cudaGetErrorString(e));
    }
    return EG_OK;
}

extern "C" int eg_host_free(void *p) {
    if (!p) return EG_OK;
    EG_CUDA(cudaFreeHost(p));
    return EG_OK;
}

extern "C" int eg_close(eg_ctx *c) {
    if (!c) return EG_OK;
    if (c->live_graphs > 0) return eg_fail(EG_EINVAL, "eg_close: %d graphs are still open", c->live_graphs);
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    cudaStreamSynchronize(c->copy_stream);
    cudaEventDestroy(c->ev0);
    cudaEventDestroy(c->ev1);
    for (cudaEvent_t e : c->evk) cudaEventDestroy(e);
    for (cudaEvent_t e : c->ev_out) cudaEventDestroy(e);
    cudaFreeHost(c->h_pinned);
    cudaStreamDestroy(c->copy_stream);
    cudaStreamDestroy(c->stream);
    delete c;
    return EG_OK;
}

extern "C" void *eg_stream(eg_ctx *c) { return c ? (void *)c->stream : nullptr; }
extern "C" int eg_sync(eg_ctx *c) {
    if (!c) return eg_fail(EG_EINVAL, "eg_sync: NULL context");
    EG_CUDA(cudaStreamSynchronize(c->stream));
    return EG_OK;
}
extern "C" uint64_t eg_bytes_in_use(eg_ctx *c) { return c ? c->in_use : 0; }
extern "C" uint64_t eg_kernel_launches(eg_ctx *c) { return c ? c->launches : 0; }

int eg_dmalloc(eg_ctx *c, void **p, uint64_t bytes) {
    *p = nullptr;
    if (bytes == 0) return EG_OK;
    if (c->budget && c->in_use + bytes > c->budget)
        return eg_fail(EG_ENOMEM, "HBM budget exceeded: %llu in use + %llu requested > %llu",
                       (unsigned long long)c->in_use, (unsigned long long)bytes, (unsigned long long)c->budget);
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return eg_fail(EG_ENOMEM, "cudaMalloc(%llu): %s", (unsigned long long)bytes, cudaGetErrorString(e));
    }
    c->in_use += bytes;
    return EG_OK;
}
void eg_dfree(eg_ctx *c, void *p, uint64_t bytes) {
    if (!p) return;
    cudaFree(p);
    c->in_use -= bytes;
}
int eg_buf_ensure(eg_ctx *c, eg_buf &b, uint64_t bytes) {
    if (b.bytes >= bytes && b.p) return EG_OK;
    eg_buf_free(c, b);
    // pad so that vector loads past the logical end stay inside the allocation
    uint64_t padded = (bytes + 255) & ~(uint64_t)255;
    padded += 256;
    EG_TRY(eg_dmalloc(c, &b.p, padded));
    b.bytes = padded;
    return EG_OK;
}
void eg_buf_free(eg_ctx *c, eg_buf &b) {
    if (b.p) eg_dfree(c, b.p, b.bytes);
    b.p = nullptr;
    b.bytes = 0;
}

// ============================================================== generators
// RMAT quadrant thresholds floor(p * 2^32) for p = .57, .76, .95.
#define RMAT_TA 2448131358u
#define RMAT_TAB 3264175144u
#define RMAT_TABC 4080218931u

__global__ void k_gen_rmat(uint32_t *pairs, uint64_t m, int scale, uint64_t seed) {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += stride) {
        uint64_t key = eg_key(seed, e);
        uint32_t s = 0, d = 0;
        uint64_t w = 0;
        for (int l = 0; l < scale; l++) {
            if ((l & 1) == 0) w = eg_draw(key, (uint64_t)(l >> 1));
            uint32_t r = (l & 1) ? (uint32_t)(w >> 32) : (uint32_t)w;
            uint32_t bit = 1u << (scale - 1 - l);
            if (r >= RMAT_TA) {
                if (r < RMAT_TAB) d |= bit;
                else if (r < RMAT_TABC) s |= bit;
                else { s |= bit; d |= bit; }
            }
        }
        reinterpret_cast<uint2 *>(pairs)[e] = make_uint2(s, d);
    }
}

__global__ void k_gen_er(uint32_t *pairs, uint64_t m, uint32_t n, uint64_t seed) {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += stride) {
        uint64_t w = eg_draw(eg_key(seed, e), 0);
        uint32_t s = (uint32_t)(((w & 0xffffffffull) * (uint64_t)n) >> 32);
        uint32_t d = (uint32_t)(((w >> 32) * (uint64_t)n) >> 32);
        reinterpret_cast<uint2 *>(pairs)[e] = make_uint2(s, d);
    }
}

static int graph_alloc(eg_ctx *ctx, uint64_t m, uint32_t n, unsigned flags, eg_graph **out) {
    if (!ctx || !out) return eg_fail(EG_EINVAL, "NULL context or output");
    *out = nullptr;
    if (n == 0) return eg_fail(EG_EINVAL, "n must be > 0");
    uint64_t M = (flags & EG_UNDIRECTED) ? 2 * m : m;
    if (M >= 0xffffffffull) return eg_fail(EG_EINVAL, "m=%llu adjacency entries: 32-bit offsets hold < 2^32",
                                            (unsigned long long)M);
    if (n == 0xffffffffu) return eg_fail(EG_EINVAL, "n must be < 2^32-1");
    eg_graph *g = new eg_graph();
    g->ctx = ctx;
    ctx->live_graphs++;
    g->n = n;
    g->m_in = m;
    g->m = M;
    g->flags = flags;
    g->built = 0;
    g->grid_p = 0;
    int rc = eg_buf_ensure(ctx, g->pairs, 2 * m * sizeof(uint32_t));
    if (rc != EG_OK) {
        ctx->live_graphs--;
        delete g;
        return rc;
    }
    *out = g;
    return EG_OK;
}

extern "C" int eg_graph_from_pairs(eg_ctx *ctx, const uint32_t *pairs, uint64_t m, uint32_t n, unsigned flags,
                                   eg_graph **out) {
    if (m && !pairs) return eg_fail(EG_EINVAL, "pairs is NULL");
    EG_TRY(graph_alloc(ctx, m, n, flags, out));
    eg_graph *g = *out;
    if (m) {
        cudaError_t e = cudaMemcpyAsync(g->pairs.p, pairs, 2 * m * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            eg_graph_free(g);
            *out = nullptr;
            return eg_fail(EG_ECUDA, "pairs H2D: %s", cudaGetErrorString(e));
        }
    }
    return EG_OK;
}

extern "C" int eg_graph_from_device_pairs(eg_ctx *ctx, const uint32_t *d_pairs, uint64_t m, uint32_t n,
                                          unsigned flags, eg_graph **out) {
    if (m && !d_pairs) return eg_fail(EG_EINVAL, "d_pairs is NULL");
    EG_TRY(graph_alloc(ctx, m, n, flags, out));
    eg_graph *g = *out;
    if (m) EG_CUDA(cudaMemcpyAsync(g->pairs.p, d_pairs, 2 * m * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->stream));
    return EG_OK;
}

extern "C" int eg_graph_from_file(eg_ctx *ctx, const char *path, uint32_t n, unsigned flags, eg_graph **out) {
    if (!path) return eg_fail(EG_EINVAL, "path is NULL");
    FILE *f = fopen(path, "rb");
    if (!f) return eg_fail(EG_EIO, "cannot open %s", path);
    struct stat sb;
    if (fstat(fileno(f), &sb) != 0) {
        fclose(f);
        return eg_fail(EG_EIO, "cannot stat %s", path);
    }
    const uint64_t rec = (flags & EG_WEIGHTED_FILE) ? 12 : 8;  // bytes per record
    if ((uint64_t)sb.st_size % rec != 0) {
        fclose(f);
        return eg_fail(EG_EIO, "%s: size %lld is not a multiple of %d bytes", path, (long long)sb.st_size, (int)rec);
    }
    uint64_t m = (uint64_t)sb.st_size / rec;
    int rc = graph_alloc(ctx, m, n, flags, out);
    if (rc != EG_OK) {
        fclose(f);
        return rc;
    }
    eg_graph *g = *out;
    // stream the file through the pinned staging (short of its readback flag
    // word); 12-byte records are compacted to [src][dst] pairs in place
    // (pair i lands at 8i <= 12i)
    const uint64_t per = EG_RB_FLAG_OFF / rec;  // records per piece
    uint64_t done = 0;
    while (done < m) {
        const uint64_t cnt = m - done < per ? m - done : per;
        const size_t got = fread(ctx->h_pinned, 1, (size_t)(cnt * rec), f);
        if (got != cnt * rec) {
            fclose(f);
            eg_graph_free(g);
            *out = nullptr;
            return eg_fail(EG_EIO, "%s: short read", path);
        }
        if (rec == 12) {
            unsigned char *b = (unsigned char *)ctx->h_pinned;
            for (uint64_t i = 0; i < cnt; i++) memmove(b + 8 * i, b + 12 * i, 8);
        }
        cudaError_t e = cudaMemcpyAsync((char *)g->pairs.p + done * 8, ctx->h_pinned, cnt * 8, cudaMemcpyHostToDevice,
                                        ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            fclose(f);
            eg_graph_free(g);
            *out = nullptr;
            return eg_fail(EG_ECUDA, "file H2D: %s", cudaGetErrorString(e));
        }
        done += cnt;
    }
    fclose(f);
    return EG_OK;
}

static uint32_t grid_for(eg_ctx *ctx, uint64_t work) {
    uint64_t b = (work + 255) / 256;
    uint64_t cap = (uint64_t)ctx->sm_count * 16;
    if (b > cap) b = cap;
    if (b == 0) b = 1;
    return (uint32_t)b;
}

extern "C" int eg_graph_generate_rmat(eg_ctx *ctx, int scale, uint64_t m, uint64_t seed, unsigned flags,
                                      eg_graph **out) {
    if (scale < 1 || scale > 31) return eg_fail(EG_EINVAL, "scale %d out of [1,31]", scale);
    EG_TRY(graph_alloc(ctx, m, 1u << scale, flags, out));
    eg_graph *g = *out;
    if (m) {
        k_gen_rmat<<<grid_for(ctx, m), 256, 0, ctx->stream>>>(bp<uint32_t>(g->pairs), m, scale, seed);
        EG_LAUNCHED(ctx);
    }
    return EG_OK;
}

extern "C" int eg_graph_generate_er(eg_ctx *ctx, uint32_t n, uint64_t m, uint64_t seed, unsigned flags,
                                    eg_graph **out) {
    EG_TRY(graph_alloc(ctx, m, n, flags, out));
    eg_graph *g = *out;
    if (m) {
        k_gen_er<<<grid_for(ctx, m), 256, 0, ctx->stream>>>(bp<uint32_t>(g->pairs), m, n, seed);
        EG_LAUNCHED(ctx);
    }
    return EG_OK;
}

extern "C" void eg_graph_free(eg_graph *g) {
    if (!g) return;
    eg_ctx *c = g->ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    eg_buf *bufs[] = {&g->pairs,        &g->csr.ptr,     &g->csr.col,        &g->csc.ptr,      &g->csc.col,
                      &g->csr.rid,      &g->csc.rid,     &g->csc_p.ptr,      &g->csc_p.col,    &g->csc_p.rid,
                      &g->perm,         &g->deg_p,       &g->csc_p_starts,   &g->csc_p_trow,
                      &g->out_deg,      &g->in_deg,      &g->cell_ptr,       &g->gsrc,         &g->gdst,
                      &g->rank,    &g->contrib0,     &g->contrib1,
                      &g->pr_part,      &g->pr_stats,    &g->mp_carry,    &g->errflag,     &g->rank_p,    &g->rank_q,    &g->level,          &g->parent,       &g->dist,
                      &g->level_s[0],   &g->level_s[1],  &g->level_s[2],  &g->parent_s[0], &g->parent_s[1],
                      &g->parent_s[2],   &g->first_in,    &g->sb.ptr,      &g->sb.rid,      &g->sb.col,
                      &g->sb.perm,       &g->sb.vals,     &g->sb.yerr,     &g->sbp.ptr,     &g->sbp.rid,
                      &g->sbp.col,       &g->sbp.perm,    &g->sbp.vals,    &g->sbp.yerr,    &g->pr_acc,
                      &g->label,        &g->spmv_x,      &g->spmv_y,      &g->spmv_vals,      &g->bfs_work,     &g->msbfs_work,
                      &g->sssp_work,    &g->ppr_work,    &g->wts,
                      &g->grid_order,   &g->grid_units,  &g->grid_off,    &g->grid_vals,   &g->grid_acc,
                      &g->esrc,         &g->edst,        &g->edge_work,
                      &g->pcol.dst,     &g->pcol.ridx,  &g->pcol.crun,   &g->pcol.rsrc,   &g->pcol.seg,
                      &g->pcol.acc,     &g->pcol.ticket,  &g->wcc_list};
    for (eg_buf *b : bufs) eg_buf_free(c, *b);
    for (eg_bfs_graph &bg : g->bfsg) {
        if (bg.exec) cudaGraphExecDestroy(bg.exec);
        if (bg.graph) cudaGraphDestroy(bg.graph);
    }
    for (eg_bfs_graph *bg : {&g->prg, &g->msg, &g->ssg, &g->ppg}) {
        if (bg->exec) cudaGraphExecDestroy(bg->exec);
        if (bg->graph) cudaGraphDestroy(bg->graph);
    }
    c->live_graphs--;
    delete g;
}

// ============================================================== scan
namespace {
constexpr int SCAN_T = 256, SCAN_I = 16, SCAN_TILE = SCAN_T * SCAN_I;

// Block-wide exclusive scan of one value per thread; returns the total.
__device__ __forceinline__ uint32_t block_exscan(uint32_t v, uint32_t &excl, uint32_t *sh /*>= 33*/) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(EG_FULL_MASK, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
        uint32_t w = lane < nw ? sh[lane] : 0;
        uint32_t s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(EG_FULL_MASK, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) sh[lane] = s - w;
        if (lane == nw - 1) sh[32] = s;
    }
    __syncthreads();
    excl = x - v + sh[warp];
    uint32_t total = sh[32];
    __syncthreads();
    return total;
}

__global__ void k_scan_reduce(const uint32_t *in, uint64_t len, uint32_t *sums) {
    __shared__ uint32_t sh[33];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_I; i++) {
        uint64_t idx = base + (uint64_t)i * SCAN_T + threadIdx.x;
        if (idx < len) s += in[idx];
    }
    uint32_t ex;
    uint32_t tot = block_exscan(s, ex, sh);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// Each thread scans SCAN_I consecutive items (loaded through shared memory).
__global__ void k_scan_apply(const uint32_t *in, uint64_t len, const uint32_t *offs, uint32_t *out, int write_total) {
    __shared__ uint32_t tile[SCAN_TILE];
    __shared__ uint32_t sh[33];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    for (int i = 0; i < SCAN_I; i++) {
        int k = i * SCAN_T + threadIdx.x;
        uint64_t idx = base + k;
        tile[k] = idx < len ? in[idx] : 0;
    }
    __syncthreads();
    uint32_t loc[SCAN_I];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_I; i++) {
        loc[i] = s;
        s += tile[threadIdx.x * SCAN_I + i];
    }
    uint32_t ex;
    uint32_t tot = block_exscan(s, ex, sh);
    uint32_t off = (offs ? offs[blockIdx.x] : 0) + ex;
#pragma unroll
    for (int i = 0; i < SCAN_I; i++) tile[threadIdx.x * SCAN_I + i] = off + loc[i];
    __syncthreads();
    for (int i = 0; i < SCAN_I; i++) {
        int k = i * SCAN_T + threadIdx.x;
        uint64_t idx = base + k;
        if (idx < len) out[idx] = tile[k];
    }
    if (write_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
        out[len] = (offs ? offs[blockIdx.x] : 0) + tot;
}
}  // namespace

int eg_exscan_u32(eg_ctx *ctx, const uint32_t *in, uint32_t *out, uint64_t len) {
    if (len == 0) {
        EG_CUDA(cudaMemsetAsync(out, 0, sizeof(uint32_t), ctx->stream));
        return EG_OK;
    }
    uint32_t nb = eg_div_up(len, SCAN_TILE);
    if (nb == 1) {
        k_scan_apply<<<1, SCAN_T, 0, ctx->stream>>>(in, len, nullptr, out, 1);
        EG_LAUNCHED(ctx);
        return EG_OK;
    }
    uint32_t *sums = nullptr;
    EG_TRY(eg_dmalloc(ctx, (void **)&sums, (uint64_t)(nb + 1) * sizeof(uint32_t)));
    k_scan_reduce<<<nb, SCAN_T, 0, ctx->stream>>>(in, len, sums);
    EG_LAUNCHED(ctx);
    int rc = eg_exscan_u32(ctx, sums, sums, nb);  // in-place is safe: one block reads all before writing
    if (rc == EG_OK) {
        k_scan_apply<<<nb, SCAN_T, 0, ctx->stream>>>(in, len, sums, out, 1);
        ctx->launches++;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = eg_fail(EG_ECUDA, "scan apply: %s", cudaGetErrorString(e));
    }
    // free after the stream has consumed it
    cudaStreamSynchronize(ctx->stream);
    eg_dfree(ctx, sums, (uint64_t)(nb + 1) * sizeof(uint32_t));
    return rc;
}

// ============================================================== histogram
__global__ void k_histogram(const uint32_t *keys, uint64_t len, uint32_t *hist) {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t start = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    // uniform trip count per warp so __match_any_sync sees full warps
    uint64_t lanes0 = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u);
    for (uint64_t i = start, w0 = lanes0; w0 < len; i += stride, w0 += stride) {
        bool valid = i < len;
        uint32_t k = valid ? keys[i] : 0xffffffffu;
        uint32_t peers = __match_any_sync(EG_FULL_MASK, k);
        if (valid && (eg_lanemask_lt() & peers) == 0) atomicAdd(&hist[k], __popc(peers));
    }
}

int eg_histogram(eg_ctx *ctx, const uint32_t *keys, uint64_t len, uint32_t *hist) {
    if (len == 0) return EG_OK;
    k_histogram<<<grid_for(ctx, len), 256, 0, ctx->stream>>>(keys, len, hist);
    EG_LAUNCHED(ctx);
    return EG_OK;
}

// ============================================================== radix sort
// Stable LSD radix sort, up to 8 bits per pass.  Per pass:
//  1. k_rs_count: per-tile digit histogram -> counts[digit][tile]
//  2. exclusive scan over counts (digit-major, tiles in order)
//  3. k_rs_scatter: stable rank of every key inside its tile (warps take
//     contiguous sub-tiles; __match_any_sync groups equal digits of a
//     32-key chunk), staging through shared memory so the global writes are
//     runs of consecutive addresses.
namespace {
constexpr int RS_T = 256, RS_I = 16, RS_TILE = RS_T * RS_I, RS_W = RS_T / 32, RS_BINS = 256;

__global__ void __launch_bounds__(RS_T) k_rs_count(const uint32_t *keys, uint64_t len, int shift, uint32_t mask,
                                                  uint32_t ntiles, uint32_t *counts) {
    __shared__ uint32_t hist[RS_BINS];
    hist[threadIdx.x] = 0;
    __syncthreads();
    uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int i = 0; i < RS_I; i++) {
        uint64_t idx = base + (uint64_t)i * RS_T + threadIdx.x;
        bool valid = idx < len;
        uint32_t d = valid ? (keys[idx] >> shift) & mask : 0xffffffffu;
        uint32_t peers = __match_any_sync(EG_FULL_MASK, d);
        if (valid && (eg_lanemask_lt() & peers) == 0) atomicAdd(&hist[d], __popc(peers));
    }
    __syncthreads();
    if (threadIdx.x <= mask) counts[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = hist[threadIdx.x];
}

__global__ void __launch_bounds__(RS_T) k_rs_scatter(const uint32_t *kin, const uint32_t *vin, uint32_t *kout,
                                                    uint32_t *vout, uint64_t len, int shift, uint32_t mask,
                                                    uint32_t ntiles, const uint32_t *offs) {
    __shared__ uint32_t wcnt[RS_W][RS_BINS];
    __shared__ uint32_t loc[RS_BINS];
    __shared__ uint32_t glob[RS_BINS];
    __shared__ uint32_t sh[33];
    __shared__ uint32_t sk[RS_TILE];
    __shared__ uint32_t sv[RS_TILE];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_W * RS_BINS; i += RS_T) (&wcnt[0][0])[i] = 0;
    __syncthreads();
    const uint64_t tile0 = (uint64_t)blockIdx.x * RS_TILE;
    const uint64_t base = tile0 + (uint64_t)warp * (RS_I * 32);
    const uint32_t lt = eg_lanemask_lt();
    uint32_t k[RS_I], v[RS_I], r[RS_I], dg[RS_I];
#pragma unroll
    for (int i = 0; i < RS_I; i++) {
        uint64_t idx = base + (uint64_t)i * 32 + lane;
        bool valid = idx < len;
        k[i] = valid ? kin[idx] : 0u;
        v[i] = valid ? vin[idx] : 0u;
        dg[i] = valid ? (k[i] >> shift) & mask : (uint32_t)RS_BINS;
    }
#pragma unroll
    for (int i = 0; i < RS_I; i++) {
        uint32_t d = dg[i];
        uint32_t peers = __match_any_sync(EG_FULL_MASK, d);
        uint32_t below = __popc(peers & lt);
        uint32_t cur = d < RS_BINS ? wcnt[warp][d] : 0u;
        r[i] = cur + below;
        __syncwarp();
        if (d < RS_BINS && below == 0) wcnt[warp][d] = cur + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        const int d = threadIdx.x;  // RS_T == RS_BINS
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < RS_W; w++) {
            uint32_t c = wcnt[w][d];
            wcnt[w][d] = run;
            run += c;
        }
        uint32_t ex;
        block_exscan(run, ex, sh);
        loc[d] = ex;
        glob[d] = (uint32_t)d <= mask ? offs[(uint64_t)d * ntiles + blockIdx.x] : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < RS_I; i++) {
        uint32_t d = dg[i];
        if (d < RS_BINS) {
            uint32_t pos = loc[d] + wcnt[warp][d] + r[i];
            sk[pos] = k[i];
            sv[pos] = v[i];
        }
    }
    __syncthreads();
    const uint32_t valid_count = (uint32_t)((len - tile0) < (uint64_t)RS_TILE ? (len - tile0) : (uint64_t)RS_TILE);
    for (uint32_t s = threadIdx.x; s < valid_count; s += RS_T) {
        uint32_t key = sk[s];
        uint32_t d = (key >> shift) & mask;
        uint32_t gpos = glob[d] + (s - loc[d]);
        kout[gpos] = key;
        vout[gpos] = sv[s];
    }
}
}  // namespace

int eg_radix_sort(eg_ctx *ctx, uint32_t *k_in, uint32_t *v_in, uint32_t *k_tmp, uint32_t *v_tmp, uint64_t len,
                  int bits, uint32_t **k_out, uint32_t **v_out) {
    *k_out = k_in;
    *v_out = v_in;
    if (len <= 1 || bits <= 0) return EG_OK;
    int passes = (bits + 7) / 8;
    int per = (bits + passes - 1) / passes;
    uint32_t ntiles = eg_div_up(len, RS_TILE);
    uint64_t ncount = (uint64_t)ntiles << per;
    uint32_t *counts = nullptr, *offs = nullptr;
    EG_TRY(eg_dmalloc(ctx, (void **)&counts, ncount * sizeof(uint32_t)));
    int rc = eg_dmalloc(ctx, (void **)&offs, (ncount + 1) * sizeof(uint32_t));
    if (rc != EG_OK) {
        eg_dfree(ctx, counts, ncount * sizeof(uint32_t));
        return rc;
    }
    uint32_t *ka = k_in, *va = v_in, *kb = k_tmp, *vb = v_tmp;
    for (int p = 0; p < passes && rc == EG_OK; p++) {
        int shift = p * per;
        int pb = bits - shift < per ? bits - shift : per;
        uint32_t mask = (1u << pb) - 1u;
        uint64_t nc = (uint64_t)ntiles * (mask + 1);
        k_rs_count<<<ntiles, RS_T, 0, ctx->stream>>>(ka, len, shift, mask, ntiles, counts);
        ctx->launches++;
        rc = eg_exscan_u32(ctx, counts, offs, nc);
        if (rc != EG_OK) break;
        k_rs_scatter<<<ntiles, RS_T, 0, ctx->stream>>>(ka, va, kb, vb, len, shift, mask, ntiles, offs);
        ctx->launches++;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = eg_fail(EG_ECUDA, "radix pass: %s", cudaGetErrorString(e));
        uint32_t *t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    cudaStreamSynchronize(ctx->stream);
    eg_dfree(ctx, counts, ncount * sizeof(uint32_t));
    eg_dfree(ctx, offs, (ncount + 1) * sizeof(uint32_t));
    *k_out = ka;
    *v_out = va;
    return rc;
}

// ============================================================== builders
// Unpacks the input pairs into (key, value) arrays: the file's edges in file
// order, then (undirected) the reversed copies, as preload_graph lays out
// memblock (init_all.c:81-110).  by_src selects key=src,value=dst.
__global__ void k_unpack(const uint32_t *pairs, uint64_t m_in, int undirected, uint32_t n, uint32_t *keys,
                         uint32_t *vals, uint32_t *bad) {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t M = undirected ? 2 * m_in : m_in;
    uint32_t anybad = 0;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < M; k += stride) {
        uint64_t e = k < m_in ? k : k - m_in;
        uint2 p = reinterpret_cast<const uint2 *>(pairs)[e];
        uint32_t s = k < m_in ? p.x : p.y;
        uint32_t d = k < m_in ? p.y : p.x;
        anybad |= (s >= n) | (d >= n);
        keys[k] = s;
        vals[k] = d;
    }
    if (__any_sync(EG_FULL_MASK, anybad) && (threadIdx.x & 31) == 0) atomicOr(bad, 1u);
}

static int bits_for(uint32_t n) {
    if (n <= 1) return 1;
    uint32_t x = n - 1;
    int b = 0;
    while (x) { b++; x >>= 1; }
    return b;
}

static int build_adj_pair(eg_graph *g, bool want_csc) {
    eg_ctx *ctx = g->ctx;
    const uint64_t M = g->m;
    const uint32_t n = g->n;
    eg_buf ka, va, kb, vb;
    int rc = EG_OK;
    uint32_t *ks = nullptr, *vs = nullptr;
    uint32_t *hbad = (uint32_t *)ctx->h_pinned;
    auto cleanup = [&]() {
        cudaStreamSynchronize(ctx->stream);
        eg_buf_free(ctx, ka);
        eg_buf_free(ctx, va);
        eg_buf_free(ctx, kb);
        eg_buf_free(ctx, vb);
    };
#define BTRY(x)                 \
    do {                        \
        rc = (x);               \
        if (rc != EG_OK) {      \
            cleanup();          \
            return rc;          \
        }                       \
    } while (0)
    BTRY(eg_buf_ensure(ctx, ka, (M + 1) * 4));
    BTRY(eg_buf_ensure(ctx, va, (M + 1) * 4));
    BTRY(eg_buf_ensure(ctx, kb, (M + 1) * 4));
    BTRY(eg_buf_ensure(ctx, vb, (M + 1) * 4));
    uint32_t *dbad = bp<uint32_t>(kb) + M;  // one spare word past the data
    if (cudaMemsetAsync(dbad, 0, 4, ctx->stream) != cudaSuccess) BTRY(eg_fail(EG_ECUDA, "memset"));
    if (M) {
        k_unpack<<<grid_for(ctx, M), 256, 0, ctx->stream>>>(bp<uint32_t>(g->pairs), g->m_in, (g->flags & EG_UNDIRECTED) != 0, n,
                                                           bp<uint32_t>(ka), bp<uint32_t>(va), dbad);
        ctx->launches++;
    }
    if (cudaMemcpyAsync(hbad, dbad, 4, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        BTRY(eg_fail(EG_ECUDA, "unpack: %s", cudaGetErrorString(cudaGetLastError())));
    if (*hbad) BTRY(eg_fail(EG_ERANGE, "an edge endpoint is >= n=%u", n));
    int bits = bits_for(n);
    // CSR: stable sort by src, value dst
    BTRY(eg_radix_sort(ctx, bp<uint32_t>(ka), bp<uint32_t>(va), bp<uint32_t>(kb), bp<uint32_t>(vb), M, bits, &ks, &vs));
    BTRY(eg_buf_ensure(ctx, g->out_deg, (uint64_t)n * 4));
    BTRY(eg_buf_ensure(ctx, g->csr.ptr, ((uint64_t)n + 1) * 4));
    BTRY(eg_buf_ensure(ctx, g->csr.col, M * 4 + 16));
    if (cudaMemsetAsync(g->out_deg.p, 0, (uint64_t)n * 4, ctx->stream) != cudaSuccess) BTRY(eg_fail(EG_ECUDA, "memset"));
    BTRY(eg_histogram(ctx, ks, M, bp<uint32_t>(g->out_deg)));
    BTRY(eg_exscan_u32(ctx, bp<uint32_t>(g->out_deg), bp<uint32_t>(g->csr.ptr), n));
    if (M && cudaMemcpyAsync(g->csr.col.p, vs, M * 4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
        BTRY(eg_fail(EG_ECUDA, "copy col"));
    BTRY(eg_buf_ensure(ctx, g->csr.rid, M * 4 + 16));
    if (M && cudaMemcpyAsync(g->csr.rid.p, ks, M * 4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
        BTRY(eg_fail(EG_ECUDA, "copy rid"));
    g->built |= EG_LAYOUT_CSR;
    g->first_in_src = nullptr;
    g->wcc_list_src = nullptr;
    if (want_csc) {
        // CSC: stable sort of the CSR entries by dst, value src.  The sorted
        // src keys become the values; the CSR cols (a copy) become the keys.
        // The temporaries are the buffer pair that does not hold the result.
        uint32_t *k2 = vs, *v2 = ks;
        uint32_t *kt = (ks == bp<uint32_t>(ka)) ? bp<uint32_t>(kb) : bp<uint32_t>(ka);
        uint32_t *vt = (ks == bp<uint32_t>(ka)) ? bp<uint32_t>(vb) : bp<uint32_t>(va);
        BTRY(eg_radix_sort(ctx, k2, v2, kt, vt, M, bits, &ks, &vs));
        BTRY(eg_buf_ensure(ctx, g->in_deg, (uint64_t)n * 4));
        BTRY(eg_buf_ensure(ctx, g->csc.ptr, ((uint64_t)n + 1) * 4));
        BTRY(eg_buf_ensure(ctx, g->csc.col, M * 4 + 16));
        if (cudaMemsetAsync(g->in_deg.p, 0, (uint64_t)n * 4, ctx->stream) != cudaSuccess) BTRY(eg_fail(EG_ECUDA, "memset"));
        BTRY(eg_histogram(ctx, ks, M, bp<uint32_t>(g->in_deg)));
        BTRY(eg_exscan_u32(ctx, bp<uint32_t>(g->in_deg), bp<uint32_t>(g->csc.ptr), n));
        if (M && cudaMemcpyAsync(g->csc.col.p, vs, M * 4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
            BTRY(eg_fail(EG_ECUDA, "copy col"));
        BTRY(eg_buf_ensure(ctx, g->csc.rid, M * 4 + 16));
        if (M && cudaMemcpyAsync(g->csc.rid.p, ks, M * 4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
            BTRY(eg_fail(EG_ECUDA, "copy rid"));
        g->built |= EG_LAYOUT_CSC;
        g->first_in_src = nullptr;
        g->wcc_list_src = nullptr;
        g->relabeled = false;  // so do PageRank's relabelled copy
        g->sb.blocks = 0;  // the source-blocked copies follow the CSC
        g->sb.shift = 0;
        g->sbp.blocks = 0;
        g->sbp.shift = 0;
    }
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        BTRY(eg_fail(EG_ECUDA, "build: %s", cudaGetErrorString(cudaGetLastError())));
#undef BTRY
    cleanup();
    return EG_OK;
}

extern "C" int eg_graph_build(eg_graph *g, unsigned layouts) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    eg_ctx *ctx = g->ctx;
    EG_CUDA(cudaSetDevice(ctx->device));
    unsigned need = layouts & ~g->built;
    EG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    if (need & (EG_LAYOUT_CSR | EG_LAYOUT_CSC)) {
        // the CSC sort consumes the CSR sort's output; rebuilding both is
        // simplest when only the CSC is missing
        EG_TRY(build_adj_pair(g, (layouts & EG_LAYOUT_CSC) != 0 || (g->built & EG_LAYOUT_CSC)));
    }
    if (need & EG_LAYOUT_GRID) {
        uint32_t P = (uint32_t)((g->n * 8u / 1024u) / 20u);  // random.c:69-71
        if (P > 2000) P = 256;
        if (P == 0) P = 4;
        EG_TRY(eg_graph_build_grid(g, P));
    }
    EG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    EG_CUDA(cudaEventSynchronize(ctx->ev1));
    EG_CUDA(cudaEventElapsedTime(&g->build_ms, ctx->ev0, ctx->ev1));
    return EG_OK;
}

// ---------------------------------------------------------------- grid
// Partition id of the reference (init_all.c:54-60, sizes from 838-842).
__device__ __forceinline__ uint32_t part_of(uint32_t v, uint32_t psz, uint32_t mod, uint32_t split) {
    if (mod == 0) return v / psz;
    return v < split ? v / psz : (v - split) / (psz - 1) + mod;
}

__global__ void k_grid_keys(const uint32_t *csr_ptr, const uint32_t *csr_col, uint32_t n, uint32_t P, uint32_t psz,
                            uint32_t mod, uint32_t split, uint32_t *cell, uint32_t *pos) {
    // one warp per source row; lanes walk the row
    uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t lane = threadIdx.x & 31;
    for (uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += warps) {
        uint32_t pu = part_of(u, psz, mod, split);
        uint32_t b = csr_ptr[u], e = csr_ptr[u + 1];
        for (uint32_t p = b + lane; p < e; p += 32) {
            cell[p] = pu * P + part_of(csr_col[p], psz, mod, split);
            pos[p] = p;
        }
    }
}

__global__ void k_csr_rows(const uint32_t *csr_ptr, uint32_t n, uint32_t *rows) {
    uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t lane = threadIdx.x & 31;
    for (uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += warps)
        for (uint32_t p = csr_ptr[u] + lane; p < csr_ptr[u + 1]; p += 32) rows[p] = u;
}

__global__ void k_grid_gather(const uint32_t *pos, const uint32_t *rows, const uint32_t *csr_col, uint64_t M,
                              uint32_t *gsrc, uint32_t *gdst) {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < M; i += stride) {
        uint32_t p = pos[i];
        gsrc[i] = rows[p];
        gdst[i] = csr_col[p];
    }
}

extern "C" int eg_graph_build_grid(eg_graph *g, uint32_t P) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    if (P == 0 || P > 4096 || P > g->n) return eg_fail(EG_EINVAL, "grid P=%u must be in [1, min(4096, n)]", P);
    eg_ctx *ctx = g->ctx;
    // The grid is built from the directed file edges (grid modes ignore -u,
    // init_all.c:636 doubles nb_edges only in init_adj_sort).
    if (g->flags & EG_UNDIRECTED) return eg_fail(EG_EINVAL, "grid layout is built from directed input (no -u)");
    if (!(g->built & EG_LAYOUT_CSR)) EG_TRY(eg_graph_build(g, EG_LAYOUT_CSR));
    const uint64_t M = g->m;
    const uint32_t n = g->n;
    uint32_t mod = n % P;
    uint32_t psz = mod ? n / P + 1 : n / P;
    uint32_t split = mod * psz;
    uint64_t cells = (uint64_t)P * P;
    eg_buf ka, va, kb, vb, rows, chist;
    int rc = EG_OK;
    auto cleanup = [&]() {
        cudaStreamSynchronize(ctx->stream);
        eg_buf_free(ctx, ka);
        eg_buf_free(ctx, va);
        eg_buf_free(ctx, kb);
        eg_buf_free(ctx, vb);
        eg_buf_free(ctx, rows);
        eg_buf_free(ctx, chist);
    };
#define GTRY(x)            \
    do {                   \
        rc = (x);          \
        if (rc != EG_OK) { \
            cleanup();     \
            return rc;     \
        }                  \
    } while (0)
    GTRY(eg_buf_ensure(ctx, ka, (M + 1) * 4));
    GTRY(eg_buf_ensure(ctx, va, (M + 1) * 4));
    GTRY(eg_buf_ensure(ctx, kb, (M + 1) * 4));
    GTRY(eg_buf_ensure(ctx, vb, (M + 1) * 4));
    GTRY(eg_buf_ensure(ctx, rows, (M + 1) * 4));
    uint32_t blocks = grid_for(ctx, (uint64_t)n * 32);
    k_grid_keys<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csr.ptr), bp<uint32_t>(g->csr.col), n, P, psz, mod,
                                                split, bp<uint32_t>(ka), bp<uint32_t>(va));
    ctx->launches++;
    k_csr_rows<<<blocks, 256, 0, ctx->stream>>>(bp<uint32_t>(g->csr.ptr), n, bp<uint32_t>(rows));
    ctx->launches++;
    uint32_t *ks, *vs;
    GTRY(eg_radix_sort(ctx, bp<uint32_t>(ka), bp<uint32_t>(va), bp<uint32_t>(kb), bp<uint32_t>(vb), M,
                       bits_for((uint32_t)cells), &ks, &vs));
    GTRY(eg_buf_ensure(ctx, g->gsrc, M * 4 + 16));
    GTRY(eg_buf_ensure(ctx, g->gdst, M * 4 + 16));
    GTRY(eg_buf_ensure(ctx, g->cell_ptr, (cells + 1) * 4));
    if (M) {
        k_grid_gather<<<grid_for(ctx, M), 256, 0, ctx->stream>>>(vs, bp<uint32_t>(rows), bp<uint32_t>(g->csr.col), M,
                                                                bp<uint32_t>(g->gsrc), bp<uint32_t>(g->gdst));
        ctx->launches++;
    }
    // cell sizes -> offsets
    GTRY(eg_buf_ensure(ctx, chist, (cells + 1) * 4));
    if (cudaMemsetAsync(chist.p, 0, cells * 4, ctx->stream) != cudaSuccess) GTRY(eg_fail(EG_ECUDA, "memset"));
    GTRY(eg_histogram(ctx, ks, M, bp<uint32_t>(chist)));
    GTRY(eg_exscan_u32(ctx, bp<uint32_t>(chist), bp<uint32_t>(g->cell_ptr), cells));
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        GTRY(eg_fail(EG_ECUDA, "grid build: %s", cudaGetErrorString(cudaGetLastError())));
#undef GTRY
    cleanup();
    g->grid_p = P;
    g->built |= EG_LAYOUT_GRID;
    g->grid_order_p = 0;  // cell order and edge values follow the new cells
    g->grid_vals_kind = 0;
    return EG_OK;
}

// ---------------------------------------------------------------- relabelled CSC
// Ascending key: vertices with in-edges first, then descending out-degree;
// ties keep ascending id (stable sort).  `rows` counts the vertices with
// in-edges, so the rows of the relabelled CSC that have entries are [0, rows).
__global__ void k_relabel_keys(const uint32_t *__restrict__ deg, const uint32_t *__restrict__ in_deg, uint32_t n,
                               uint32_t *keys, uint32_t *vals, uint32_t *rows) {
    uint32_t cnt = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t d = deg[v] < 0x7fffffffu ? deg[v] : 0x7fffffffu;
        const bool in = in_deg[v] != 0;
        keys[v] = (in ? 0u : 0x80000000u) | (0x7fffffffu - d);
        vals[v] = v;
        cnt += in;
    }
    cnt = __reduce_add_sync(EG_FULL_MASK, cnt);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(rows, cnt);
}
__global__ void k_relabel_perm(const uint32_t *__restrict__ order, const uint32_t *__restrict__ deg, uint32_t n,
                               uint32_t *perm, uint32_t *deg_p) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t old = order[i];
        perm[old] = i;
        deg_p[i] = deg[old];
    }
}
// CSC entry (row v, column u) -> (key perm[u], value perm[v])
__global__ void k_relabel_entries(const uint32_t *__restrict__ rid, const uint32_t *__restrict__ col,
                                  const uint32_t *__restrict__ perm, uint64_t m, uint32_t *keys, uint32_t *vals) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        keys[e] = perm[col[e]];
        vals[e] = perm[rid[e]];
    }
}

// Row-start bits of the relabelled CSC: bit e of word e/32 is set when entry
// e begins a row (its row differs from entry e-1's); words past the entries
// are 0.  One warp per word, the bits from a ballot.
__global__ void k_row_starts(const uint32_t *__restrict__ rid, uint64_t m, uint64_t nbits, uint32_t *starts) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;  // a multiple of 32: warps stay whole
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nbits; e += stride) {
        const bool s = e < m && (e == 0 || rid[e] != rid[e - 1]);
        const uint32_t b = __ballot_sync(EG_FULL_MASK, s);
        if ((threadIdx.x & 31) == 0) starts[e >> 5] = b;
    }
}
// Row of every EG_TROW_SPAN-th entry.
__global__ void k_trow(const uint32_t *__restrict__ rid, uint64_t m, uint32_t *trow) {
    const uint64_t nt = (m + EG_TROW_SPAN - 1) / EG_TROW_SPAN;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += (uint64_t)gridDim.x * blockDim.x)
        trow[i] = rid[i * EG_TROW_SPAN];
}

int eg_build_relabeled_csc(eg_graph *g) {
    if (g->relabeled) return EG_OK;
    if (!(g->built & EG_LAYOUT_CSC) || !(g->built & EG_LAYOUT_CSR))
        return eg_fail(EG_ENOTBUILT, "relabelled CSC needs the CSC and the out-degrees");
    g->pcol.shift = 0;  // the partition layout is made from this copy
    eg_ctx *ctx = g->ctx;
    const uint32_t n = g->n;
    const uint64_t M = g->m;
    eg_buf ka, va, kb, vb;
    int rc = EG_OK;
    auto cleanup = [&]() {
        cudaStreamSynchronize(ctx->stream);
        eg_buf_free(ctx, ka);
        eg_buf_free(ctx, va);
        eg_buf_free(ctx, kb);
        eg_buf_free(ctx, vb);
    };
#define RTRY(x)            \
    do {                   \
        rc = (x);          \
        if (rc != EG_OK) { \
            cleanup();     \
            return rc;     \
        }                  \
    } while (0)
    const uint64_t len = M > n ? M : n;
    RTRY(eg_buf_ensure(ctx, ka, (len + 1) * 4));
    RTRY(eg_buf_ensure(ctx, va, (len + 1) * 4));
    RTRY(eg_buf_ensure(ctx, kb, (len + 1) * 4));
    RTRY(eg_buf_ensure(ctx, vb, (len + 1) * 4));
    RTRY(eg_buf_ensure(ctx, g->perm, (uint64_t)n * 4));
    RTRY(eg_buf_ensure(ctx, g->deg_p, (uint64_t)n * 4));
    uint32_t *ks, *vs;
    // the count of rows with entries goes to the word after the key array
    // (the buffers hold len + 1 words; the sorts use the first n)
    uint32_t *rows_dev = bp<uint32_t>(kb) + len;
    if (cudaMemsetAsync(rows_dev, 0, 4, ctx->stream) != cudaSuccess) RTRY(eg_fail(EG_ECUDA, "memset"));
    k_relabel_keys<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(bp<uint32_t>(g->out_deg), bp<uint32_t>(g->in_deg), n,
                                                             bp<uint32_t>(ka), bp<uint32_t>(va), rows_dev);
    ctx->launches++;
    uint32_t rows_host = 0;
    if (cudaMemcpyAsync(&rows_host, rows_dev, 4, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        RTRY(eg_fail(EG_ECUDA, "relabel count"));
    RTRY(eg_radix_sort(ctx, bp<uint32_t>(ka), bp<uint32_t>(va), bp<uint32_t>(kb), bp<uint32_t>(vb), n, 32, &ks, &vs));
    k_relabel_perm<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(vs, bp<uint32_t>(g->out_deg), n, bp<uint32_t>(g->perm),
                                                             bp<uint32_t>(g->deg_p));
    ctx->launches++;
    // entries in the new ids: stable sort by new src, then by new dst
    if (M) {
        k_relabel_entries<<<grid_for(ctx, M), 256, 0, ctx->stream>>>(bp<uint32_t>(g->csc.rid), bp<uint32_t>(g->csc.col),
                                                                    bp<uint32_t>(g->perm), M, bp<uint32_t>(ka),
                                                                    bp<uint32_t>(va));
        ctx->launches++;
    }
    const int bits = n <= 1 ? 1 : 32 - __builtin_clz(n - 1);
    RTRY(eg_radix_sort(ctx, bp<uint32_t>(ka), bp<uint32_t>(va), bp<uint32_t>(kb), bp<uint32_t>(vb), M, bits, &ks, &vs));
    uint32_t *kt = (ks == bp<uint32_t>(ka)) ? bp<uint32_t>(kb) : bp<uint32_t>(ka);
    uint32_t *vt = (ks == bp<uint32_t>(ka)) ? bp<uint32_t>(vb) : bp<uint32_t>(va);
    RTRY(eg_radix_sort(ctx, vs, ks, kt, vt, M, bits, &ks, &vs));  // keys: new dst, values: new src
    RTRY(eg_buf_ensure(ctx, g->csc_p.ptr, ((uint64_t)n + 1) * 4));
    RTRY(eg_buf_ensure(ctx, g->csc_p.col, M * 4 + 16));
    RTRY(eg_buf_ensure(ctx, g->csc_p.rid, M * 4 + 16));
    if (M) {
        if (cudaMemcpyAsync(g->csc_p.col.p, vs, M * 4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess ||
            cudaMemcpyAsync(g->csc_p.rid.p, ks, M * 4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
            RTRY(eg_fail(EG_ECUDA, "relabel copy"));
    }
    // row pointers from the row histogram (reuse kb/vb: no longer needed)
    uint32_t *hist = bp<uint32_t>(ka);  // stream order: the copies above have read ks/vs first
    if (cudaMemsetAsync(hist, 0, (uint64_t)n * 4, ctx->stream) != cudaSuccess) RTRY(eg_fail(EG_ECUDA, "memset"));
    RTRY(eg_histogram(ctx, bp<uint32_t>(g->csc_p.rid), M, hist));
    RTRY(eg_exscan_u32(ctx, hist, bp<uint32_t>(g->csc_p.ptr), n));
    // row-start bits and the row of every 512th entry: with the rows that
    // have entries numbered 0 .. rows-1, they give every entry's row
    const uint64_t nwords = (M + 31) / 32 + EG_STARTS_PAD;
    RTRY(eg_buf_ensure(ctx, g->csc_p_starts, nwords * 4));
    RTRY(eg_buf_ensure(ctx, g->csc_p_trow, ((M + EG_TROW_SPAN - 1) / EG_TROW_SPAN + 1) * 4));
    k_row_starts<<<grid_for(ctx, nwords * 32), 256, 0, ctx->stream>>>(bp<uint32_t>(g->csc_p.rid), M, nwords * 32,
                                                                      bp<uint32_t>(g->csc_p_starts));
    ctx->launches++;
    if (M) {
        k_trow<<<grid_for(ctx, (M + EG_TROW_SPAN - 1) / EG_TROW_SPAN), 256, 0, ctx->stream>>>(
            bp<uint32_t>(g->csc_p.rid), M, bp<uint32_t>(g->csc_p_trow));
        ctx->launches++;
    }
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        RTRY(eg_fail(EG_ECUDA, "relabel: %s", cudaGetErrorString(cudaGetLastError())));
#undef RTRY
    cleanup();
    g->relabeled = true;
    g->csc_p_rows = rows_host;
    return EG_OK;
}

// ============================================================== queries
extern "C" int eg_graph_get_info(eg_graph *g, eg_graph_info *info) {
    if (!g || !info) return eg_fail(EG_EINVAL, "NULL argument");
    info->n = g->n;
    info->m_input = g->m_in;
    info->m = g->m;
    info->layouts = g->built;
    info->grid_p = g->grid_p;
    info->device_bytes = g->ctx->in_use;
    info->build_ms = g->build_ms;
    return EG_OK;
}

extern "C" int eg_graph_copy_adj(eg_graph *g, unsigned layout, uint32_t *ptr, uint32_t *col) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    eg_adj *a = layout == EG_LAYOUT_CSR ? &g->csr : layout == EG_LAYOUT_CSC ? &g->csc : nullptr;
    if (!a) return eg_fail(EG_EINVAL, "layout must be EG_LAYOUT_CSR or EG_LAYOUT_CSC");
    if (!(g->built & layout)) return eg_fail(EG_ENOTBUILT, "layout %u not built", layout);
    eg_ctx *ctx = g->ctx;
    if (ptr) EG_CUDA(cudaMemcpyAsync(ptr, a->ptr.p, ((uint64_t)g->n + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (col && g->m) EG_CUDA(cudaMemcpyAsync(col, a->col.p, g->m * 4, cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    return EG_OK;
}

extern "C" int eg_graph_copy_grid(eg_graph *g, uint32_t *cell_ptr, uint32_t *src, uint32_t *dst) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    if (!(g->built & EG_LAYOUT_GRID)) return eg_fail(EG_ENOTBUILT, "grid not built");
    eg_ctx *ctx = g->ctx;
    uint64_t cells = (uint64_t)g->grid_p * g->grid_p;
    if (cell_ptr) EG_CUDA(cudaMemcpyAsync(cell_ptr, g->cell_ptr.p, (cells + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (src && g->m) EG_CUDA(cudaMemcpyAsync(src, g->gsrc.p, g->m * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (dst && g->m) EG_CUDA(cudaMemcpyAsync(dst, g->gdst.p, g->m * 4, cudaMemcpyDeviceToHost, ctx->stream));
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    return EG_OK;
}

extern "C" int eg_graph_copy_degrees(eg_graph *g, uint32_t *out_deg, uint32_t *in_deg) {
    if (!g) return eg_fail(EG_EINVAL, "NULL graph");
    eg_ctx *ctx = g->ctx;
    if (out_deg) {
        if (!(g->built & (EG_LAYOUT_CSR | EG_LAYOUT_EDGES))) return eg_fail(EG_ENOTBUILT, "CSR not built");
        EG_CUDA(cudaMemcpyAsync(out_deg, g->out_deg.p, (uint64_t)g->n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (in_deg) {
        if (!(g->built & (EG_LAYOUT_CSC | EG_LAYOUT_EDGES))) return eg_fail(EG_ENOTBUILT, "CSC not built");
        EG_CUDA(cudaMemcpyAsync(in_deg, g->in_deg.p, (uint64_t)g->n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    EG_CUDA(cudaStreamSynchronize(ctx->stream));
    return EG_OK;
}

extern "C" void *eg_graph_device_ptr(eg_graph *g, int which) {
    if (!g) return nullptr;
    switch (which) {
        case EG_DEV_CSR_PTR: return g->csr.ptr.p;
        case EG_DEV_CSR_COL: return g->csr.col.p;
        case EG_DEV_CSC_PTR: return g->csc.ptr.p;
        case EG_DEV_CSC_COL: return g->csc.col.p;
        case EG_DEV_OUT_DEG: return g->out_deg.p;
        case EG_DEV_EDGE_SRC: return g->esrc.p;
        case EG_DEV_EDGE_DST: return g->edst.p;
        case EG_DEV_RANK: return g->rank.p;
        case EG_DEV_LEVEL: return g->level.p;
        case EG_DEV_PARENT: return g->parent.p;
        case EG_DEV_DIST: return g->dist.p;
        case EG_DEV_LABEL: return g->label.p;
        case EG_DEV_SPMV_Y: return g->spmv_y.p;
        default: return nullptr;
    }
}

extern "C" int eg_sample_roots(eg_graph *g, int k, uint64_t seed, uint32_t *roots_out) {
    if (!g || !roots_out || k < 0) return eg_fail(EG_EINVAL, "bad argument");
    if (!(g->built & EG_LAYOUT_CSR)) return eg_fail(EG_ENOTBUILT, "CSR not built");
    uint32_t n = g->n;
    uint32_t *deg = (uint32_t *)malloc((size_t)n * 4);
    if (!deg) return eg_fail(EG_ENOMEM, "host malloc");
    int rc = eg_graph_copy_degrees(g, deg, nullptr);
    if (rc != EG_OK) {
        free(deg);
        return rc;
    }
    for (int i = 0; i < k; i++) {
        uint64_t key = eg_key(seed, (uint64_t)i);
        int found = 0;
        for (uint64_t a = 0; a < (1u << 20); a++) {
            uint32_t v = (uint32_t)(((eg_draw(key, a) >> 32) * (uint64_t)n) >> 32);
            if (deg[v] > 0) {
                roots_out[i] = v;
                found = 1;
                break;
            }
        }
        if (!found) {
            free(deg);
            return eg_fail(EG_EINVAL, "no vertex with positive out-degree");
        }
    }
    free(deg);
    return EG_OK;
}
