// Batched pairwise set intersection.
//
// BATCHED (RTG_SI_AUTO): one persistent kernel streams every pair through a per-warp ring of
// shared-memory slots filled by 1-D bulk copies (cp.async.bulk, one mbarrier per slot).
// A pair whose lists fit one slot is one job. A longer pair is cut into K chunks of each
// list (K = ceil((|A|+|B|) / slot capacity)); its jobs are the chunk pairs (p, q) whose
// value ranges overlap, visited in merge order from the chunk maxima (loaded lane-parallel),
// so every common element lies in exactly one job. Inside a slot every lane takes 1/32 of
// the merged sequence (merge-path split point by binary search) and merges serially,
// counting a common element when its B copy is consumed right after an equal A element.
// Lists are read once from HBM in large asynchronous copies, several jobs in flight per
// warp.
//
// Per-family kernel (PLAIN and the forced families): warps take 32 pairs at a time from an
// atomic queue; lane i loads the ids and list bounds of pair i, then the warp intersects
// the pairs one after another straight from global memory:
//   MERGE  – warp tile merge, both lists streamed (balanced lengths),
//   SEARCH – short-list elements binary-searched in the long list (skewed lengths),
//   HASH   – short list hashed into the warp's shared-memory table, long list streamed
//            through it (the block-bitmap / hash-table baselines' formulation).
// PLAIN picks SEARCH when |long| > ratio * |short|, MERGE otherwise.
//
// Counts are exact set-intersection sizes: what the reference's kernels accumulate per
// (A_i, B_j) with atomics (set_intersection/baseline/bs.cu:138-209, hi.cu:134-181,
// ip.cu:138-287, bi_dynamic.cu:134-169) and what its Check compares against the
// generator's known overlap (set_intersection/utils/util.cpp:39-51).
#include <cub/cub.cuh>

#include <algorithm>

#include "internal.h"
#include "intersect.cuh"
#include "tma.cuh"

namespace rtg {

namespace {

constexpr uint32_t kDefaultSiWarps = 8;
constexpr uint32_t kDefaultSearchRatio = 32;
constexpr uint32_t kSiHashSlots = 2048;
constexpr uint32_t kDefaultStreamWarps = 8;
constexpr uint32_t kDefaultStageSlots = 2;
constexpr uint32_t kDefaultStageBytes = 4096;

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
    if (f == RTG_SI_PLAIN) f = ((uint64_t)b > (uint64_t)ratio * a) ? RTG_SI_FORCE_SEARCH : RTG_SI_FORCE_MERGE;
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

// ---------------------------------------------------------------- batched form

struct StreamCfg {
    uint32_t S;           // staging slots per warp
    uint32_t slot_words;  // 32-bit words per slot
    uint32_t meta_off;    // byte offsets of the shared-memory regions
    uint32_t ring_off;
};

constexpr uint32_t kMetaWords = 8;  // per slot: A offset, |A part|, B offset, |B part|, pair, last

// Count |A ∩ B| of two sorted unique lists in shared memory: lane l merges diagonals
// [l*L/32, (l+1)*L/32) of the merged sequence (ties take A first) and counts an element of
// B when it equals the A element consumed just before it.
__device__ __forceinline__ uint32_t merge_path_count(const uint32_t *A, uint32_t na,
                                                     const uint32_t *B, uint32_t nb, int lane) {
    const uint32_t L = na + nb;
    const uint32_t d0 = (uint32_t)(((uint64_t)L * (uint32_t)lane) >> 5);
    const uint32_t d1 = (uint32_t)(((uint64_t)L * (uint32_t)(lane + 1)) >> 5);
    uint32_t lo = d0 > nb ? d0 - nb : 0u, hi = min(d0, na);
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (A[mid] <= B[d0 - 1 - mid]) lo = mid + 1;
        else hi = mid;
    }
    uint32_t i = lo, j = d0 - lo;
    uint32_t last = i ? A[i - 1] : kEmpty;
    uint32_t ai = i < na ? A[i] : kEmpty, bj = j < nb ? B[j] : kEmpty;
    uint32_t c = 0;
    for (uint32_t d = d0; d < d1; ++d) {
        if (i < na && (j >= nb || ai <= bj)) {
            last = ai;
            ++i;
            ai = i < na ? A[i] : kEmpty;
        } else {
            c += (bj == last) ? 1u : 0u;
            ++j;
            bj = j < nb ? B[j] : kEmpty;
        }
    }
    return c;
}

__global__ void k_si_stream(SiArgs s, uint32_t *out, unsigned long long *head, StreamCfg p,
                            uint32_t *status) {
    extern __shared__ __align__(128) unsigned char stage_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t *bars = reinterpret_cast<uint64_t *>(stage_smem) + (size_t)warp * p.S;
    uint32_t *meta =
        reinterpret_cast<uint32_t *>(stage_smem + p.meta_off) + (size_t)warp * p.S * kMetaWords;
    uint32_t *ring =
        reinterpret_cast<uint32_t *>(stage_smem + p.ring_off) + (size_t)warp * p.S * p.slot_words;
    if ((uint32_t)lane < p.S) mbar_init(bars + lane, 1);
    fence_mbar_init();
    __syncwarp();
    const uint32_t CAPE = p.slot_words - 16;  // list elements per job (room for alignment)

    // producer: batches of 32 pairs, the next batch fetched one batch ahead
    auto fetch = [&](unsigned long long &base, PairRef &r) {
        unsigned long long b0 = 0;
        if (lane == 0) b0 = atomicAdd(head, 32ull);
        base = __shfl_sync(kFull, b0, 0);
        const uint64_t k = base + lane;
        const bool in = k < s.np;
        r = load_pair(s, k, in);
        if (in && !r.valid) {
            atomicExch(status, kStatusBadInput);
            out[k] = 0;
        }
    };
    unsigned long long cb, nb;
    PairRef cr, nr;
    fetch(cb, cr);
    fetch(nb, nr);
    uint32_t e = 0;
    // the pair being cut into jobs (warp-uniform)
    bool open = false;
    uint64_t oa = 0, ob = 0, pk = 0;
    uint32_t a = 0, b = 0, CA = 0, CB = 0, KA = 0, KB = 0, pA = 0, qB = 0, wA = 0, wB = 0;
    uint32_t mxA = kEmpty, mxB = kEmpty;  // lane t: largest element of chunk wA+t / wB+t
    auto chunk_max = [&](uint32_t w, uint32_t K, uint32_t C, uint64_t o, uint32_t len) {
        const uint32_t t = w + lane;
        return t < K ? __ldg(s.elems + o + min((t + 1) * C, len) - 1) : kEmpty;
    };
    auto next_job = [&](uint32_t &a0, uint32_t &na, uint32_t &b0, uint32_t &nbb, bool &last) {
        while (!open) {
            if (cb >= s.np) return false;
            if (e >= 32 || cb + e >= s.np) {
                cb = nb;
                cr = nr;
                e = 0;
                if (cb < s.np) fetch(nb, nr);
                continue;
            }
            const bool valid = __shfl_sync(kFull, cr.valid ? 1u : 0u, e) != 0u;
            oa = __shfl_sync(kFull, cr.oa, e);
            ob = __shfl_sync(kFull, cr.ob, e);
            a = __shfl_sync(kFull, cr.a, e);
            b = __shfl_sync(kFull, cr.b, e);
            pk = cb + e;
            ++e;
            if (!valid) continue;
            if (a == 0) {  // a <= b: an empty list meets nothing
                if (lane == 0) out[pk] = 0;
                continue;
            }
            if ((uint64_t)a + b <= CAPE) {
                CA = a;
                CB = b;
                KA = KB = 1;
            } else {
                const uint32_t K = (uint32_t)(((uint64_t)a + b + CAPE - 1) / CAPE);
                CA = (a + K - 1) / K;
                CB = (b + K - 1) / K;
                KA = (a + CA - 1) / CA;
                KB = (b + CB - 1) / CB;
                mxA = chunk_max(0, KA, CA, oa, a);
                mxB = chunk_max(0, KB, CB, ob, b);
            }
            pA = qB = wA = wB = 0;
            open = true;
        }
        a0 = pA * CA;
        na = min(CA, a - a0);
        b0 = qB * CB;
        nbb = min(CB, b - b0);
        if (KA == 1 && KB == 1) {
            last = true;
            open = false;
            return true;
        }
        // next chunk pair in merge order of the chunk maxima
        const uint32_t ma = __shfl_sync(kFull, mxA, pA - wA), mb = __shfl_sync(kFull, mxB, qB - wB);
        if (ma <= mb) ++pA;
        if (mb <= ma) ++qB;
        last = pA >= KA || qB >= KB;
        if (last) {
            open = false;
        } else {
            if (pA - wA >= 32) {
                wA += 32;
                mxA = chunk_max(wA, KA, CA, oa, a);
            }
            if (qB - wB >= 32) {
                wB += 32;
                mxB = chunk_max(wB, KB, CB, ob, b);
            }
        }
        return true;
    };

    uint32_t inflight = 0, sw = 0, sr = 0, phase = 0, acc = 0;
    bool jobs = true;
    while (true) {
        while (inflight < p.S && jobs) {
            uint32_t a0, na, b0, nbb;
            bool last;
            if (!next_job(a0, na, b0, nbb, last)) {
                jobs = false;
                break;
            }
            const uintptr_t ga = reinterpret_cast<uintptr_t>(s.elems + oa + a0);
            const uintptr_t gb = reinterpret_cast<uintptr_t>(s.elems + ob + b0);
            const uintptr_t gaa = ga & ~(uintptr_t)15, gbb = gb & ~(uintptr_t)15;
            const uint32_t hA = (uint32_t)(ga - gaa) >> 2, hB = (uint32_t)(gb - gbb) >> 2;
            const uint32_t bytesA = ((hA + na) * 4u + 15u) & ~15u;
            const uint32_t bytesB = ((hB + nbb) * 4u + 15u) & ~15u;
            uint32_t *slot = ring + (size_t)sw * p.slot_words;
            if (lane == 0) {
                uint32_t *mt = meta + sw * kMetaWords;
                mt[0] = hA;
                mt[1] = na;
                mt[2] = bytesA / 4 + hB;
                mt[3] = nbb;
                mt[4] = (uint32_t)pk;
                mt[5] = last ? 1u : 0u;
                mbar_arrive_expect_tx(bars + sw, bytesA + bytesB);
                bulk_copy_g2s(slot, reinterpret_cast<const void *>(gaa), bytesA, bars + sw);
                bulk_copy_g2s(slot + bytesA / 4, reinterpret_cast<const void *>(gbb), bytesB,
                              bars + sw);
            }
            sw = (sw + 1 == p.S) ? 0 : sw + 1;
            ++inflight;
        }
        if (inflight == 0) break;
        __syncwarp();
        if (!mbar_wait(bars + sr, (phase >> sr) & 1u)) {
            if (lane == 0) atomicExch(status, kStatusTimeout);
            for (uint32_t q = 1; q < inflight; ++q) {  // bounded drain of the others
                const uint32_t s2 = (sr + q) % p.S;
                mbar_wait(bars + s2, (phase >> s2) & 1u);
            }
            break;
        }
        phase ^= 1u << sr;
        const uint32_t *mt = meta + sr * kMetaWords;
        const uint32_t *slot = ring + (size_t)sr * p.slot_words;
        uint32_t c = merge_path_count(slot + mt[0], mt[1], slot + mt[2], mt[3], lane);
        c = __reduce_add_sync(kFull, c);
        acc += c;
        if (mt[5]) {
            if (lane == 0) out[mt[4]] = acc;
            acc = 0;
        }
        __syncwarp();
        fence_proxy_async_smem();
        sr = (sr + 1 == p.S) ? 0 : sr + 1;
        --inflight;
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
    if (family == RTG_SI_AUTO) {
        const rtg_config &cf = ctx->cfg;
        const uint32_t W = cf.si_block_warps ? cf.si_block_warps : kDefaultStreamWarps;
        StreamCfg sc{};
        sc.S = cf.si_stage_slots ? cf.si_stage_slots : kDefaultStageSlots;
        const uint32_t slot_bytes = cf.si_stage_bytes ? cf.si_stage_bytes : kDefaultStageBytes;
        sc.slot_words = slot_bytes / 4;
        sc.meta_off = ((W * sc.S * 8) + 127u) & ~127u;
        sc.ring_off = (sc.meta_off + W * sc.S * kMetaWords * 4 + 127u) & ~127u;
        const size_t smem = (size_t)sc.ring_off + (size_t)W * sc.S * slot_bytes;
        if ((int)smem > ctx->smem_optin)
            return fail(ctx, RTG_ERR_INVALID_ARG, "SI schedule needs %zu B of shared memory", smem);
        RTG_CUDA(ctx, cudaFuncSetAttribute(k_si_stream, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
        int per_sm = 0;
        RTG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_si_stream, W * 32, smem));
        if (cf.si_blocks_per_sm) per_sm = std::min<int>(per_sm, (int)cf.si_blocks_per_sm);
        per_sm = std::max(per_sm, 1);
        const uint64_t need = (ps.npairs + 32ull * W - 1) / (32ull * W);
        const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)ctx->sm_count * per_sm));
        unsigned long long *head = ctx->d_scalars + 8;
        RTG_CUDA(ctx, cudaMemsetAsync(head, 0, 8, ctx->stream));
        RTG_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
        k_si_stream<<<grid, W * 32, smem, ctx->stream>>>(make_args(ps), d_out, head, sc,
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
