// =============================================================================
// agg_lane.cuh -- the "lane block" pair task of the single-instance aggregation
// kernel on geometric grids: one output slot per lane, the lags split over the
// CTA's warps, and the larger member's factor taken out of each run of lags
// with the same bracket offset.
//
// Slot sums as in agg_tile.cuh: slot s collects the pairs (j, k = j + d) whose
// bracket is lo = s, R_s = sum rate, TH_s = sum rate (fl(x_j + x_k) - x_s) 2^St_s
// (reference src/aggregation_kernels.cuh:145-239, regrouped). On a verified
// geometric grid lo(j, j + d) = j + Ld[d], so slot s meets lag d in the pair
// j = s - Ld[d], k = s - e(d) with e(d) = Ld[d] - d >= 0. e is the same for
// every slot, and it stays constant over runs of consecutive lags (Ld grows by
// one per lag once the pivot ratio makes x_0 + x_d fall in the bin above x_d;
// e = 0, the lags whose pairs land on their larger member, is one long run).
// Within a run, k is fixed per slot, so for every kernel but Sum
//   rate = F_k q(d, j),   F = N (x N for Product), q = B_d N_j + S_d x_j N_j,
// and a lane sums q and q th over the run and multiplies by F_k once:
// 3 FP64 instructions per pair for one-term kernels, 4 for Brownian + shear
// (the tile task needs 5 where lo > k). Sum keeps its per-pair rate.
//
// Work split: blocks of 32 output bins aligned to the top of the grid (block
// t owns bins [n - 32 (t + 1), n - 32 t), as the tiles do, so bin n - 1 is never
// a block's first bin); a task is one block and one chunk of C lags; the CTA's
// eight warps take equal contiguous shares of the chunk's lags (each warp sees
// its runs in order) and their sums are added in warp order. A block with
// several chunk tasks stores each chunk's 2 x 32 sums; the block's last task
// (ticket) adds them in chunk order and writes the bins -- deterministic,
// nobody waits.
//
// Operand staging (template STAGE): the j-side operands of a task (N_j,
// x_j N_j, x_j for j in one contiguous window of at most kLaneWinMax entries)
// are copied into shared memory with bulk TMA copies (cp.async.bulk, mbarrier
// completion); without STAGE the lanes read them through the read-only cache.
// =============================================================================
#pragma once

#include <cstdint>

#include "agg_tile.cuh"

namespace pbe_gb300 {

constexpr int kLaneWarps = kMainThreads / 32;       // warps sharing a task's lags
constexpr int kLaneWinMax = 1792;                   // staged window, entries per array (even)
// Bounded waits on the staging barrier: iterations of mbarrier.try_wait.
constexpr long long kLaneWaitLimit = 1LL << 26;

// Index of task (block t, chunk c): the tasks of chunk c' < c come first.
__device__ __forceinline__ int lane_task_index(int n, int t, int c, int C)
{
    int base = 0;
    for (int q = 0; q < c; ++q) base += lane_chunk_blocks(n, q, C);
    return base + t;
}

// ---- bulk TMA copy + mbarrier helpers (shared::cta addresses) -----------------
__device__ __forceinline__ unsigned smem_addr(const void* p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
// Waits for the barrier's phase `parity` to complete; false after kLaneWaitLimit tries.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity)
{
    const unsigned a = smem_addr(bar);
    for (long long it = 0; it < kLaneWaitLimit; ++it) {
        unsigned done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Shared memory of a lane task (carved from the kernel's dynamic buffer).
struct LaneSmem {
    double* red;     // [kLaneWarps][2][32] per-warp R, TH
    double* wN;      // [kLaneWinMax] staged N_j   (K needs N on the j side)
    double* wH;      // [kLaneWinMax] staged x_j N_j
    double* wX;      // [kLaneWinMax] staged x_j
};

// Staged copies of N and x (scratch, 256-byte aligned, at least n + 2 entries)
// and the chunk partials / tickets of the lane path.
struct LaneArgs {
    const double* Ncp;   // N copy
    const double* xcp;   // x copy
    double* part;        // [lane_partial_doubles(n)]
    int* ticket;         // [lane_blocks(n)] chunk tasks of the block done (reset by the prep)
    int* err;            // set to 1 when a staging wait gave up
    int C;               // lag chunk length
};

// One lane task: block t, lag chunk c. All kMainThreads threads of the CTA
// take part; returns with the CTA synchronised. `phase` is the staging
// barrier's parity (flipped per staged task). Gather mode stores / finishes
// the block's bins; scatter mode flushes this chunk's share with atomics.
template <int K, bool SCATTER, bool STAGE>
__device__ void lane_task(const AggCellView& v, const AggWs& ws, const LaneArgs& la, double* rhs,
                          int t, int c, int nclip, const LaneSmem& sm, uint64_t* bar,
                          unsigned& phase, int* s_flag)
{
    const int n = v.n;
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int C = la.C;
    const int I = n - kLaneBins * (t + 1);
    const int smax = lane_block_smax(n, t);
    const int smin = I > 0 ? I : 0;
    const int nch = lane_block_chunks(n, t, C);

    // lags of this task: [dA, dB), dB cut where Ld passes the block's top slot
    // (Ld is nondecreasing; clipped lags hold kLagClipAll)
    const int dA = c * C;
    int dB = min(dA + C, smax + 1);
    // most chunks end below the cut: one load settles it, else bisect
    if (dB > dA && __ldg(v.Ld + dB - 1) > smax) {
        int lo = dA, hi = dB;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(v.Ld + mid) > smax) hi = mid; else lo = mid + 1;
        }
        dB = lo;
    }

    // j-side operand pointers: the staged window or the arrays themselves
    const double* pN = v.Nj;
    const double* pH = v.Hj;
    const double* pX = v.x;
    int jw0 = 0;
    if (STAGE && dB > dA) {
        jw0 = smin - __ldg(v.Ld + dB - 1);
        jw0 = jw0 > 0 ? (jw0 & ~1) : 0;
        int jw1 = smax - __ldg(v.Ld + dA) + 1;        // exclusive, <= n - 1
        jw1 = (jw1 + 1) & ~1;                          // <= n: copies are padded
        const int cnt = jw1 - jw0;
        if (cnt > 0 && cnt <= kLaneWinMax) {
            const unsigned bytes = static_cast<unsigned>(cnt) * 8u;
            if (tid == 0) {
                fence_proxy_async_smem();              // earlier generic reads of the window
                mbar_expect_tx(bar, (NeedH<K>::j ? 3u : 2u) * bytes);
                bulk_g2s(sm.wN, la.Ncp + jw0, bytes, bar);
                if constexpr (NeedH<K>::j) bulk_g2s(sm.wH, v.Hj + jw0, bytes, bar);
                bulk_g2s(sm.wX, la.xcp + jw0, bytes, bar);
            }
            if (!mbar_wait(bar, phase)) {
                // the copy never completed: flag it, poison the block's bins, leave
                if (tid == 0) *la.err = 1;
                *s_flag = 1;
            }
            phase ^= 1u;
            pN = sm.wN - jw0;
            pH = sm.wH - jw0;
            pX = sm.wX - jw0;
        }
    }

    // this warp's contiguous share of the lags
    const int len = dB - dA;
    const int per = (len + kLaneWarps - 1) / kLaneWarps;
    const int dw0 = dA + w * per;
    const int dw1 = min(dB, dw0 + per);

    const int s = I + lane;
    const bool slot = (s >= smin && s <= smax);
    const double xs = slot ? __ldg(v.x + s) : 0.0;
    const int St = slot ? -ilogb(xs) : 0;
    const EwOperandC pc = ew_operand_c(xs, St);       // the slot pivot, decoded once
    EwOperandA pa = ew_operand_a(0.0);                // x_k of the current run
    double R = 0.0, TH = 0.0, Q = 0.0, QT = 0.0;
    double F = 0.0, xk = 0.0, Nk = 0.0, hk = 0.0;
    int e_cur = -1;
    if (!*s_flag) {
        for (int d = dw0; d < dw1; ++d) {
            const int L = __ldg(v.Ld + d);
            const int e = L - d;
            if (e != e_cur) {                          // uniform across the warp
                if constexpr (K != 1) {
                    R = fma(F, Q, R);
                    TH = fma(F, QT, TH);
                    Q = 0.0;
                    QT = 0.0;
                }
                e_cur = e;
                const int k = s - e;
                const bool kin = slot && k >= 0;
                F = kin ? __ldg(v.Fs + k) : 0.0;
                xk = kin ? __ldg(v.x + k) : 0.0;
                pa = ew_operand_a(xk);
                if constexpr (K == 1) {
                    Nk = kin ? __ldg(v.Nk + k) : 0.0;
                    hk = kin ? __ldg(v.Hk + k) : 0.0;
                }
            }
            const double B = __ldg(v.Bd + d), S = __ldg(v.Sd + d);
            const int j = s - L;
            if (slot && j >= 0) {
                const double Nj = pN[j];
                const double hj = NeedH<K>::j ? pH[j] : 0.0;
                const double th = sum_minus_scaled_pre(pa, pX[j], pc);
                if constexpr (K != 1) {
                    const double q = q_slot<K>(B, S, Nj, hj);
                    Q += q;
                    QT = fma(q, th, QT);
                } else {
                    const double rate = rate_geo<1>(B, S, Nj, hj, Nk, hk);
                    R += rate;
                    TH = fma(rate, th, TH);
                }
            }
        }
        if constexpr (K != 1) {
            R = fma(F, Q, R);
            TH = fma(F, QT, TH);
        }
    }
    sm.red[(w * 2 + 0) * 32 + lane] = R;
    sm.red[(w * 2 + 1) * 32 + lane] = TH;
    __syncthreads();
    const bool poisoned = *s_flag != 0;

    if (w == 0) {
        double Rt = 0.0, THt = 0.0;
#pragma unroll
        for (int q = 0; q < kLaneWarps; ++q) {
            Rt += sm.red[(q * 2 + 0) * 32 + lane];
            THt += sm.red[(q * 2 + 1) * 32 + lane];
        }
        bool finish = true;
        if (!SCATTER && nch > 1) {
            double* cp = la.part + static_cast<size_t>(lane_task_index(n, t, c, C)) * 64;
            cp[lane] = Rt;
            cp[32 + lane] = THt;
            __threadfence();                           // every lane's sums before the ticket
            __syncwarp();
            int last = 0;
            if (lane == 0) last = (atomicAdd(la.ticket + t, 1) == nch - 1);
            last = __shfl_sync(0xffffffffu, last, 0);
            finish = last != 0;
            if (finish) {
                __threadfence();
                Rt = 0.0;
                THt = 0.0;
                int idx = t;                           // task index of (t, q), q = 0, 1, ...
                for (int q = 0; q < nch; ++q) {
                    const double* pq = la.part + static_cast<size_t>(idx) * 64;
                    Rt += __ldcg(pq + lane);
                    THt += __ldcg(pq + 32 + lane);
                    idx += lane_chunk_blocks(n, q, C);
                }
            }
        }
        if (finish) {
            const int i = s;
            // own part of bin i (slot i) and the w-part of slot i, owed to bin i + 1
            double b1 = 0.0, co = 0.0;
            if (slot) {
                const double sd = scalbn(__ldg(v.inv_dx + i), -St);
                b1 = fma(-THt, sd, Rt);
                co = THt * sd;
            }
            const double cin = __shfl_up_sync(0xffffffffu, co, 1);
            if constexpr (SCATTER) {
                if (i >= 0) {
                    double val = b1;
                    if (lane >= 1) val += cin;
                    if (c == 0) val -= agg_death<K>(v, i);
                    if (val != 0.0) atomicAdd(rhs + i, val);
                }
                if (lane == 31 && slot && co != 0.0) atomicAdd(rhs + i + 1, co);
            } else {
                if (i >= 0) {
                    double val = b1;
                    if (lane >= 1) val += cin;
                    val -= agg_death<K>(v, i);
                    if (poisoned) val = __longlong_as_double(0x7ff8000000000000LL);
                    if (lane == 0 && I >= 1) {
                        ws.tfirst[t] = val;
                        __threadfence();
                        if (atomicAdd(ws.tticket + t, 1) == 1) {
                            __threadfence();
                            rhs[I] = __ldcg(rhs + I) + (__ldcg(ws.tfirst + t) + __ldcg(ws.tcarry + t));
                        }
                    } else {
                        rhs[i] = rhs[i] + val;
                        if (i == n - 1) {
                            __threadfence();
                            if (atomicAdd(ws.counter + 3, 1) == nclip) {
                                __threadfence();
                                double sc = 0.0;
                                for (int q = 0; q < nclip; ++q) sc += __ldcg(ws.clip_part + q);
                                rhs[n - 1] = __ldcg(rhs + (n - 1)) + sc;
                            }
                        }
                    }
                }
                if (lane == 31 && t >= 1) {
                    // carry into bin I + 32, the first bin of block t - 1
                    ws.tcarry[t - 1] = co;
                    __threadfence();
                    if (atomicAdd(ws.tticket + (t - 1), 1) == 1) {
                        __threadfence();
                        const int J = I + kLaneBins;
                        rhs[J] = __ldcg(rhs + J) + (__ldcg(ws.tfirst + t - 1) + __ldcg(ws.tcarry + t - 1));
                    }
                }
            }
        }
    }
    __syncthreads();
}

} // namespace pbe_gb300
