// Device-side validation of the CSR forms the counting kernels read.
//
// The batched triangle count indexes a per-warp bitmap by (element - window origin) and
// takes every element of a suffix range of an in-edge of v to be a rank above v; the
// per-edge forms read rows by their offsets. A form that breaks those invariants (a
// damaged cache file, a builder fault) would send a kernel out of its buffers. These
// kernels check every invariant the counting kernels rely on, reading only at indexes that
// are loop counters or values already checked against their array's size, and report a
// violation in the device status word (kStatusBadForm -> RTG_ERR_FORMAT). The checked
// build (RTG_CHECKED) runs them before every count; the host check of cache files
// (csr_cache.cpp) applies the same rules on the CPU.
#include <algorithm>

#include "internal.h"

namespace rtg {

bool g_skip_file_structure_checks = false;

namespace {

__device__ __forceinline__ void bad_form(uint32_t *status) { atomicExch(status, kStatusBadForm); }

// The last index i in [0, n] with off[i] <= x. Offsets that are not monotone give some
// index in [0, n], which the caller checks (off[i] <= x < off[i + 1]).
__device__ __forceinline__ uint32_t row_of(const uint64_t *__restrict__ off, uint32_t n,
                                           uint64_t x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo + 1) / 2;
        if (off[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// offsets: off[0] = 0, off[n] = m, non-decreasing
__global__ void k_check_offsets(const uint64_t *__restrict__ off, uint32_t n, uint64_t m,
                                uint32_t *status) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v <= n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t o = off[v];
        if ((v == 0 && o != 0) || (v == n && o != m) || (v < n && o > off[v + 1]))
            bad_form(status);
    }
}

// rows: every id below n, rows strictly ascending, and with above_vertex every id of row v
// above v. Runs after k_check_offsets on the same stream; it still only reads adj at q < m
// and off at indexes in [0, n].
__global__ void k_check_rows(const uint64_t *__restrict__ off, const uint32_t *__restrict__ adj,
                             uint32_t n, uint64_t m, bool above_vertex, uint32_t *status) {
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < m;
         q += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t w = adj[q];
        const uint32_t v = row_of(off, n, q);
        if (w >= n || v >= n || off[v] > q || q >= off[v + 1] || (above_vertex && w <= v) ||
            (q > off[v] && adj[q - 1] >= w))
            bad_form(status);
    }
}

// in-edge ranges of a counting form: in-edge e of head v (in_off[v] <= e < in_off[v + 1])
// holds [x, y) with x <= y <= m, x not below the previous in-edge's x (in-edges ordered by
// source: the dense-core split takes those from core rows to be the last ones of v); a
// non-empty range lies inside one row u of the CSR and starts at an element above v (rows
// ascend, so all of it is above v)
__global__ void k_check_ranges(const uint64_t *__restrict__ off, const uint32_t *__restrict__ adj,
                               const uint64_t *__restrict__ in_off,
                               const uint2 *__restrict__ in_rng, uint32_t n, uint64_t m,
                               uint64_t m_in, uint32_t *status) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m_in;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 r = in_rng[e];
        const uint32_t v = row_of(in_off, n, e);
        if (v >= n || in_off[v] > e || e >= in_off[v + 1] || r.x > r.y || r.y > m ||
            (e > in_off[v] && in_rng[e - 1].x > r.x)) {
            bad_form(status);
            continue;
        }
        if (r.x == r.y) continue;
        const uint32_t u = row_of(off, n, r.x);
        if (u >= n || off[u] > r.x || r.y > off[u + 1] || adj[r.x] <= v) bad_form(status);
    }
}

int grid_for(const rtg_ctx *ctx, uint64_t work) {
    return (int)std::max<uint64_t>(1, std::min<uint64_t>((work + 255) / 256, ctx->sm_count * 16ull));
}

// offsets first, then what depends on them: a form with bad offsets is refused before any
// row is read through them
rtg_status check_rows_of(rtg_ctx *ctx, const uint64_t *off, const uint32_t *adj, uint32_t n,
                         uint64_t m, bool above_vertex) {
    k_check_offsets<<<grid_for(ctx, n + 1ull), 256, 0, ctx->stream>>>(off, n, m, ctx->d_status);
    RTG_CUDA(ctx, cudaGetLastError());
    ctx->launches++;
    RTG_TRY(check_status_word(ctx));
    if (m) {
        k_check_rows<<<grid_for(ctx, m), 256, 0, ctx->stream>>>(off, adj, n, m, above_vertex,
                                                                ctx->d_status);
        RTG_CUDA(ctx, cudaGetLastError());
        ctx->launches++;
        RTG_TRY(check_status_word(ctx));
    }
    return RTG_OK;
}

}  // namespace

rtg_status check_csr(rtg_ctx *ctx, const Csr &c, bool above_vertex) {
    if (!c.built) return RTG_OK;
    return check_rows_of(ctx, c.off, c.adj, c.n, c.m, above_vertex);
}

rtg_status check_count_form(rtg_ctx *ctx, const CountCsr &cc) {
    if (!cc.built) return RTG_OK;
    RTG_TRY(check_rows_of(ctx, cc.off, cc.adj, cc.n, cc.m, true));
    // in-edge offsets end at the in-edges held (a one-shot form holds those below its core)
    const uint64_t mi = cc.inedges();
    k_check_offsets<<<grid_for(ctx, cc.n + 1ull), 256, 0, ctx->stream>>>(cc.in_off, cc.n, mi,
                                                                         ctx->d_status);
    RTG_CUDA(ctx, cudaGetLastError());
    ctx->launches++;
    RTG_TRY(check_status_word(ctx));
    if (mi) {
        k_check_ranges<<<grid_for(ctx, mi), 256, 0, ctx->stream>>>(
            cc.off, cc.adj, cc.in_off, cc.in_rng, cc.n, cc.m, mi, ctx->d_status);
        RTG_CUDA(ctx, cudaGetLastError());
        ctx->launches++;
        RTG_TRY(check_status_word(ctx));
    }
    return RTG_OK;
}

}  // namespace rtg

extern "C" int rtg_checked_build(void) { return rtg::kChecked ? 1 : 0; }

extern "C" rtg_status rtg_debug_skip_file_checks(int on) {
    if (!rtg::kChecked) return RTG_ERR_STATE;
    rtg::g_skip_file_structure_checks = on != 0;
    return RTG_OK;
}
