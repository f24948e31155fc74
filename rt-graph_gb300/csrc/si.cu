// Batched pairwise set intersection.
//
// One persistent kernel: warps take 32 pairs at a time from an atomic queue; lane i loads
// the ids and list bounds of pair i (so the dependent loads of 32 pairs overlap), then the
// warp intersects the pairs one after another with the family chosen per pair:
//   MERGE  – warp tile merge, both lists streamed (balanced lengths),
//   SEARCH – short-list elements binary-searched in the long list (skewed lengths),
//   HASH   – short list hashed into the warp's shared-memory table, long list streamed
//            through it (the block-bitmap / hash-table baselines' formulation).
// AUTO picks SEARCH when |long| > ratio * |short|, MERGE otherwise.
//
// Counts are exact set-intersection sizes: what the reference's kernels accumulate per
// (A_i, B_j) with atomics (set_intersection/baseline/bs.cu:138-209, hi.cu:134-181,
// ip.cu:138-287, bi_dynamic.cu:134-169) and what its Check compares against the
// generator's known overlap (set_intersection/utils/util.cpp:39-51).
#include <cub/cub.cuh>

#include <algorithm>

#include "internal.h"
#include "intersect.cuh"

namespace rtg {

namespace {

constexpr uint32_t kDefaultSiWarps = 8;
constexpr uint32_t kDefaultSearchRatio = 32;
constexpr uint32_t kSiHashSlots = 2048;

struct SiArgs {
    const uint64_t *off;
    const uint32_t *elems;
    uint64_t nsets;
    const uint32_t *pa;
    const uint32_t *pb;
    uint64_t np;
    uint32_t dense_nb, a_begin, b_begin;
};

__device__ __forceinline__ bool pair_ids(const SiArgs &s, uint64_t k, uint32_t &x, uint32_t &y) {
    if (s.dense_nb) {
        x = s.a_begin + (uint32_t)(k / s.dense_nb);
        y = s.b_begin + (uint32_t)(k % s.dense_nb);
    } else {
        x = __ldg(s.pa + k);
        y = __ldg(s.pb + k);
    }
    return x < s.nsets && y < s.nsets;
}

// Per-lane prefetch of one pair: pointers and lengths, short list first.
struct PairRef {
    uint64_t oa, ob;
    uint32_t a, b;
    bool valid;
};

__device__ __forceinline__ PairRef load_pair(const SiArgs &s, uint64_t k, bool in_range) {
    PairRef r{0, 0, 0, 0, false};
    if (!in_range) return r;
    uint32_t x, y;
    if (!pair_ids(s, k, x, y)) return r;
    uint64_t ox = __ldg(s.off + x), oy = __ldg(s.off + y);
    uint32_t lx = (uint32_t)(__ldg(s.off + x + 1) - ox), ly = (uint32_t)(__ldg(s.off + y + 1) - oy);
    if (lx <= ly) {
        r.oa = ox; r.a = lx; r.ob = oy; r.b = ly;
    } else {
        r.oa = oy; r.a = ly; r.ob = ox; r.b = lx;
    }
    r.valid = true;
    return r;
}

__device__ __forceinline__ uint32_t intersect_family(const uint32_t *elems, uint64_t oa, uint32_t a,
                                                     uint64_t ob, uint32_t b, uint32_t family,
                                                     uint32_t ratio, uint32_t *tab, uint32_t H,
                                                     int lane) {
    if (a == 0) return 0;
    const uint32_t *A = elems + oa, *B = elems + ob;
    uint32_t f = family;
    if (f == RTG_SI_AUTO) f = ((uint64_t)b > (uint64_t)ratio * a) ? RTG_SI_FORCE_SEARCH : RTG_SI_FORCE_MERGE;
    if (f == RTG_SI_FORCE_SEARCH) return warp_search_count(A, a, B, b, lane);
    if (f == RTG_SI_FORCE_BITMAP && a <= H / 2) {
        uint32_t lg = hash_lg_for(a);
        warp_hash_build(tab, lg, A, a, lane);
        uint32_t c = warp_hash_stream(tab, lg, B, b, lane);
        __syncwarp();
        return c;
    }
    return warp_merge_count(A, a, B, b, lane);
}

__global__ void k_si_count(SiArgs s, uint32_t *out, unsigned long long *head, uint32_t family,
                           uint32_t ratio, uint32_t H, uint32_t *status) {
    extern __shared__ __align__(16) uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t *tab = smem + warp * H;
    while (true) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(head, 32ull);
        base = __shfl_sync(kFull, base, 0);
        if (base >= s.np) break;
        const uint64_t k = base + lane;
        const bool in_range = k < s.np;
        PairRef r = load_pair(s, k, in_range);
        if (in_range && !r.valid) {
            atomicExch(status, kStatusBadInput);
            out[k] = 0;
        }
        unsigned vmask = __ballot_sync(kFull, r.valid);
        uint32_t mine = 0;
        while (vmask) {
            const int e = __ffs(vmask) - 1;
            vmask &= vmask - 1;
            const uint64_t oa = __shfl_sync(kFull, r.oa, e), ob = __shfl_sync(kFull, r.ob, e);
            const uint32_t a = __shfl_sync(kFull, r.a, e), b = __shfl_sync(kFull, r.b, e);
            uint32_t c = intersect_family(s.elems, oa, a, ob, b, family, ratio, tab, H, lane);
            c = __reduce_add_sync(kFull, c);
            if (lane == e) mine = c;
        }
        if (r.valid) out[k] = mine;
    }
}

__global__ void k_si_write(SiArgs s, const uint64_t *__restrict__ out_off, uint32_t *out_elems) {
    const int lane = threadIdx.x & 31;
    uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t k = warp; k < s.np; k += nwarps) {
        uint32_t x, y;
        if (!pair_ids(s, k, x, y)) continue;
        uint64_t ox = s.off[x], oy = s.off[y];
        uint32_t lx = (uint32_t)(s.off[x + 1] - ox), ly = (uint32_t)(s.off[y + 1] - oy);
        warp_merge_write(s.elems + ox, lx, s.elems + oy, ly, out_elems + out_off[k], lane);
    }
}

__global__ void k_widen(const uint32_t *__restrict__ in, uint64_t n, uint64_t *out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = in[i];
}

SiArgs make_args(const PairSpec &ps) {
    SiArgs a;
    a.off = ps.off;
    a.elems = ps.elems;
    a.nsets = ps.nsets;
    a.pa = ps.pa;
    a.pb = ps.pb;
    a.np = ps.npairs;
    a.dense_nb = ps.dense_nb;
    a.a_begin = ps.a_begin;
    a.b_begin = ps.b_begin;
    return a;
}

}  // namespace

rtg_status si_count_device(rtg_ctx *ctx, const PairSpec &ps, uint32_t *d_out, uint32_t family,
                           float *kernel_ms, uint64_t *launches) {
    if (ps.npairs == 0) {
        if (kernel_ms) *kernel_ms = 0;
        return RTG_OK;
    }
    const uint32_t W = ctx->cfg.si_block_warps ? ctx->cfg.si_block_warps : kDefaultSiWarps;
    const uint32_t ratio = ctx->cfg.si_search_ratio ? ctx->cfg.si_search_ratio : kDefaultSearchRatio;
    const uint32_t H = (family == RTG_SI_FORCE_BITMAP) ? kSiHashSlots : 0;
    const size_t smem = (size_t)W * H * 4;
    if ((int)smem > ctx->smem_optin)
        return fail(ctx, RTG_ERR_INVALID_ARG, "SI schedule needs %zu B of shared memory", smem);
    RTG_CUDA(ctx, cudaFuncSetAttribute(k_si_count, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)std::max<size_t>(smem, 0)));
    int per_sm = 0;
    RTG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_si_count, W * 32, smem));
    per_sm = std::max(per_sm, 1);
    uint64_t need_blocks = (ps.npairs + 32 * W - 1) / (32 * W);
    int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(need_blocks, (uint64_t)ctx->sm_count * per_sm));
    unsigned long long *head = ctx->d_scalars + 8;
    RTG_CUDA(ctx, cudaMemsetAsync(head, 0, 8, ctx->stream));
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
    k_si_count<<<grid, W * 32, smem, ctx->stream>>>(make_args(ps), d_out, head, family, ratio, H,
                                                    ctx->d_status);
    RTG_CUDA(ctx, cudaGetLastError());
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
    (*launches)++;
    if (kernel_ms) {
        RTG_CUDA(ctx, cudaEventSynchronize(ctx->ev[7]));
        cudaEventElapsedTime(kernel_ms, ctx->ev[6], ctx->ev[7]);
    }
    return RTG_OK;
}

rtg_status si_materialize_device(rtg_ctx *ctx, const PairSpec &ps, uint64_t *d_out_off,
                                 uint32_t *d_out_elems, uint64_t capacity, uint64_t *needed,
                                 uint64_t *launches) {
    const uint64_t np = ps.npairs;
    *needed = 0;
    // per-pair counts, widened to uint64, exclusive scan -> output offsets
    void *p = nullptr;
    RTG_TRY(scratch(ctx, 1, (np + 1) * 12 + 16, &p));
    uint32_t *cnt = (uint32_t *)p;
    uint64_t *wide = (uint64_t *)(((uintptr_t)(cnt + np + 1) + 15) & ~(uintptr_t)15);
    RTG_CUDA(ctx, cudaMemsetAsync(cnt, 0, (np + 1) * 4, ctx->stream));
    RTG_TRY(si_count_device(ctx, ps, cnt, RTG_SI_AUTO, nullptr, launches));
    k_widen<<<(int)std::max<uint64_t>(1, std::min<uint64_t>((np + 256) / 256, ctx->sm_count * 16ull)),
              256, 0, ctx->stream>>>(cnt, np + 1, wide);
    RTG_CUDA(ctx, cudaGetLastError());
    (*launches)++;
    size_t bytes = 0;
    RTG_CUDA(ctx, cub::DeviceScan::ExclusiveSum(nullptr, bytes, wide, d_out_off, (int64_t)np + 1,
                                                ctx->stream));
    void *tmp = nullptr;
    RTG_TRY(scratch(ctx, 0, bytes, &tmp));
    RTG_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp, bytes, wide, d_out_off, (int64_t)np + 1,
                                                ctx->stream));
    (*launches) += 2;
    uint64_t total = 0;
    RTG_CUDA(ctx, cudaMemcpyAsync(&total, d_out_off + np, 8, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *needed = total;
    if (total > capacity) return RTG_ERR_INVALID_ARG;
    if (np && total) {
        int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((np + 7) / 8, ctx->sm_count * 32ull));
        k_si_write<<<grid, 256, 0, ctx->stream>>>(make_args(ps), d_out_off, d_out_elems);
        RTG_CUDA(ctx, cudaGetLastError());
        (*launches)++;
    }
    return RTG_OK;
}

}  // namespace rtg
