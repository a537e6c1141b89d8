// Allocation-free SpMV entry point.
//
// Some callers cannot allocate device memory at all: code running inside a
// host callback or a memory-pool-constrained service, plug-ins loaded into a
// process whose allocator they do not own, or a caller that has already
// handed all of HBM to a pool.  eg_spmv_f32_noalloc serves them: the caller
// passes device pointers to its own inputs and output, and the only other
// memory the row reduction needs (the merge-path schedule and the per-CTA
// carries) lives in the fixed array below, which every GPU that loads this
// library holds until the process exits.
#include <mutex>

#include "eg_mp.cuh"

#define EG_NOALLOC_T 256
#define EG_NOALLOC_IPT 8
#define EG_NOALLOC_ITEMS (EG_NOALLOC_T * EG_NOALLOC_IPT)
#define EG_NOALLOC_MAX_TILES ((uint32_t)(EG_NOALLOC_MAX_ITEMS / EG_NOALLOC_ITEMS))

namespace {

struct NoallocScratch {
    uint2 coord[EG_NOALLOC_MAX_TILES + 1];
    eg_mp_carry<float> carry[EG_NOALLOC_MAX_TILES];
};

// 1.5 MiB per device: room for n + m <= EG_NOALLOC_MAX_TILES * 2048 items.
static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// Host-side addresses of g_noalloc_scratch, looked up once per device.
std::mutex g_noalloc_mu;
NoallocScratch *g_noalloc_addr[64];

struct NoallocSpmvOp {
    using V = float;
    using A = float;
    const float *__restrict__ x;
    const float *__restrict__ vals;  // NULL: every entry has value 1
    float *__restrict__ y;
    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void setup() {}
    __device__ __forceinline__ V gather(uint32_t j, uint32_t u) const {
        const float xv = __ldg(x + u);
        return vals ? __fmul_rn(__ldg(vals + j), xv) : xv;
    }
    __device__ __forceinline__ A zero() const { return 0.f; }
    __device__ __forceinline__ A add(A a, V v) const { return a + v; }
    __device__ __forceinline__ A merge(A a, A b) const { return a + b; }
    __device__ __forceinline__ float2 emit(uint32_t v, A s) const {
        y[v] = s;
        return make_float2(0.f, 0.f);
    }
};

int noalloc_scratch(int dev, NoallocScratch **out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (dev < 0 || dev >= 64) return eg_fail(EG_EINVAL, "device %d out of range", dev);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return eg_fail(EG_ECUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        g_noalloc_addr[dev] = (NoallocScratch *)p;
    }
    *out = g_noalloc_addr[dev];
    return EG_OK;
}

}  // namespace

extern "C" int eg_spmv_f32_noalloc(const uint32_t *d_ptr, const uint32_t *d_col, const float *d_vals,
                                   const float *d_x, float *d_y, uint32_t n, uint64_t m, void *stream) {
    if (!d_ptr || !d_x || !d_y || (m && !d_col)) return eg_fail(EG_EINVAL, "eg_spmv_f32_noalloc: NULL pointer");
    if (n == 0) return EG_OK;
    if (m >= 0xffffffffull) return eg_fail(EG_EINVAL, "m=%llu: 32-bit offsets hold < 2^32", (unsigned long long)m);
    const uint64_t items = (uint64_t)n + m;
    const uint64_t ntiles64 = (items + EG_NOALLOC_ITEMS - 1) / EG_NOALLOC_ITEMS;
    if (ntiles64 > EG_NOALLOC_MAX_TILES)
        return eg_fail(EG_EINVAL,
                       "eg_spmv_f32_noalloc: n + m = %llu exceeds the fixed scratch limit of %llu (n + m <= %d * %d)",
                       (unsigned long long)items, (unsigned long long)EG_NOALLOC_MAX_TILES * EG_NOALLOC_ITEMS,
                       EG_NOALLOC_MAX_TILES, EG_NOALLOC_ITEMS);
    const uint32_t ntiles = (uint32_t)ntiles64;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return eg_fail(EG_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    NoallocScratch *scr = nullptr;
    EG_TRY(noalloc_scratch(dev, &scr));
    cudaStream_t st = (cudaStream_t)stream;
    // Everything the kernels read from the scratch is written earlier in the
    // same call (schedule, then every CTA's carry), so nothing is cleared.
    k_mp_schedule<<<eg_div_up(ntiles + 1, 256), 256, 0, st>>>(d_ptr, n, (uint32_t)m, EG_NOALLOC_ITEMS, ntiles,
                                                             scr->coord);
    e = cudaGetLastError();
    if (e != cudaSuccess) return eg_fail(EG_ECUDA, "schedule launch: %s", cudaGetErrorString(e));
    NoallocSpmvOp op{d_x, d_vals, d_y};
    using L = eg_mp_smem<EG_NOALLOC_T, EG_NOALLOC_IPT, float, float>;
    k_mp_rows<NoallocSpmvOp, EG_NOALLOC_T, EG_NOALLOC_IPT, false>
        <<<ntiles, EG_NOALLOC_T, L::bytes, st>>>(d_ptr, d_col, n, scr->coord, scr->carry, nullptr, op);
    e = cudaGetLastError();
    if (e != cudaSuccess) return eg_fail(EG_ECUDA, "row-reduction launch: %s", cudaGetErrorString(e));
    k_mp_fixup<NoallocSpmvOp, false><<<eg_div_up((uint64_t)ntiles * 32, 256), 256, 0, st>>>(d_ptr, scr->coord, ntiles,
                                                                                         scr->carry, nullptr, op);
    e = cudaGetLastError();
    if (e != cudaSuccess) return eg_fail(EG_ECUDA, "fix-up launch: %s", cudaGetErrorString(e));
    return EG_OK;
}
