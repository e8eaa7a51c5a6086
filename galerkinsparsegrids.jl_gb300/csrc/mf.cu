// mf.cu -- the matrix-free form: one persistent launch per RK4 step (all
// four stages), or per stage for single-stage lists (operator applications,
// tile tuning).
//
// The launch walks an ordered work list (engine.h): for each group of solves
// of a class and each RK stage, one pass per dimension d.  A pass item is a
// pencil tile: the pencil's 1D prefix (m = k 2^(lmax-1) rows) times W columns
// taken across the group's solves.  The tile is gathered into shared memory
// with cp.async, swept with the 1D operator's k x k blocks (stored as FP32
// hi + lo pairs and applied with the paired FMA __ffma2_rn, so the operator
// carries ~FP64 entries while the data stays FP32), and the result is added
// into the FP32 partial-sum vector rhs (L2-resident for the group, accessed
// with .cg so other SMs' writes are seen).  For the wave (u_tt = sum_d D_d D_d u) the
// tile applies the 1D operator twice.  The last dimension's tile completes
// the right-hand side of its elements and applies the RK stage update to
// them in place: FP64 state, the stage combination, and the FP32 stage input
// of the next stage (for the wave also the displacement field, whose
// derivative is the velocity's stage input).
//
// Ordering: items are handed out in list order by an atomic counter.  A CTA
// claims its next item when the current one has passed all of its waits (at
// the start of its output, so the claim's round trip overlaps the output),
// and starts it right after that output.  An item of phase p waits (bounded
// spin) until every item of phase p-1 of its group has finished, and an item
// that gathers the stage input of stage s >= 2 first waits for its group's
// RK phase of stage s - 1; those come earlier in the list, so progress never
// depends on a later item.  A wait that runs out sets *err and the item goes
// on with what it has.
#include <cuda_runtime.h>

#include <cstddef>
#include <map>
#include <mutex>
#include <type_traits>

#include "bounds.cuh"
#include "engine.h"
#include "cvt.cuh"
#include "mf_sweep.cuh"
#include "rk.cuh"

namespace sgdg {

__device__ __forceinline__ void cp_async4(float* smem_dst, const float* gmem_src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem_src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }


__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_relaxed(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Applies the pencil's 1D operator to src for every (row block, column quad)
// of the tile and hands each result to emit(rb, jq, out).  In the
// hierarchical basis a coarse row block couples to most blocks of the pencil
// (row block 0 to all of them) while a fine one couples to O(levels), so the
// coarse rows (rb < rlong) are shared by a warp -- lanes split the block list,
// a fixed shuffle tree sums -- and the fine rows get one thread each.
template <int K, int CPT, class Emit>
__device__ __forceinline__ void apply_rows(const OpTable& T, const float* __restrict__ src, int W, int nrb, int lwq,
                                           int rlong, Emit&& emit) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nql = rlong << lwq;
    for (int u = warp; u < nql; u += kMFThreads / 32) {
        const int rb = u >> lwq, jq = u & ((1 << lwq) - 1);
        float o[K][CPT];
        sweep<K, CPT>(T, src, W, nrb, rb, jq, lane, 32, o);
        warp_sum<K, CPT>(o);
        if (lane == 0) emit(rb, jq, o);
    }
    const int nq = nrb << lwq;
    for (int q = nql + (int)threadIdx.x; q < nq; q += kMFThreads) {
        const int rb = q >> lwq, jq = q & ((1 << lwq) - 1);
        float o[K][CPT];
        sweep<K, CPT>(T, src, W, nrb, rb, jq, 0, 1, o);
        emit(rb, jq, o);
    }
}

// Waits (thread 0, bounded) until counter ctr reaches need; the caller's
// following __syncthreads publishes the outcome to the CTA.
__device__ __forceinline__ void wait_counter(const int* ctr, int need, int* err) {
    int polls = 0;
    while (ld_acquire(ctr) < need) {
        if (++polls > kSpinLimit || ld_relaxed(err) != 0) {
            atomicExch(err, 1);
            break;
        }
        __nanosleep(100);
    }
}

// Runs col(j, r0, rstep) for the columns j of a W-column tile: consecutive
// threads take consecutive columns (min(W, kMFThreads) of them), and each
// thread then walks its column's rows r0, r0 + rstep, ... (so per-column
// values are computed once per thread and a warp's accesses follow a row).
template <class ColFn>
__device__ __forceinline__ void tile_columns(int W, int lw, ColFn&& col) {
    const int cl = lw < kMFThreadsLog2 ? lw : kMFThreadsLog2;
    const int r0 = (int)threadIdx.x >> cl, rstep = kMFThreads >> cl;
    for (int j = (int)threadIdx.x & ((1 << cl) - 1); j < W; j += 1 << cl) col(j, r0, rstep);
}

// One pencil tile.  Element (row, j) of the tile lives at offset
// rinfo[row].x + ca[j] + (cb[j] << rinfo[row].y) of solve cslot[j]: the
// row part (level block, cell and mode along d) and the column part (cells
// and modes of the other dimensions, the high cell part scaled by the row
// level's cell count) are tabulated once per tile in shared memory.
constexpr int kOutRows = 4;       // rows per batch of the output loops

// FP64 state loads: from L2 (never an L1 line another SM's write left stale:
// in a whole-step launch the state was written by an earlier stage's item,
// possibly on another SM), with an evict-first L2 policy (each value is read
// once per stage).
__device__ __forceinline__ double ld_state(const double* p, unsigned long long pol) {
    double v;
    asm volatile("ld.global.cg.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
    return v;
}

template <int K, int CPT, bool WAVE, bool TWICE>
__device__ void pass_tile(const MFItem& it, const MFClass& C, const OpTable& T, int stage, int in_sel, float* smem,
                          int* ctr, int* err, int* claim, unsigned long long pol) {
    const int tid = threadIdx.x;
    const int nrb = 1 << (it.lmax - 1);
    const int m = nrb * K;
    const int W = it.W, Wv = it.Wv;
    const int lw = __ffs(W) - 1;  // W is a power of two
    int* cslot = reinterpret_cast<int*>(smem);
    int* ca = cslot + W;
    int* cb = ca + W;
    int2* rinfo = reinterpret_cast<int2*>(cb + W);              // 12W bytes in: 8-aligned (W even)
    float* X = reinterpret_cast<float*>(rinfo + ((m + 1) & ~1));  // + 8 mpad: 16-aligned for W % 4 == 0
    float* Y = X + m * W;
    const int kD = C.kD, kd1 = it.kd1, lp = it.lp, R = it.R, kDm1 = it.kDm1;
    for (int j = tid; j < W; j += kMFThreads) {
        if (j < Wv) {
            // column g of the class: slot, then (cells, modes) of the other dimensions
            const int g = it.g0 + j;
            const int slot = div_invariant(g, it.rmagic, it.rshift), r = g - slot * R;
            const int cr = div_pow<K>(r, C.D - 1), mr = r - cr * kDm1;
            const int mq = div_pow<K>(mr, it.d);
            cslot[j] = SGDG_IN(slot, C.nslots) ? slot : -1;
            ca[j] = kD * (cr & ((1 << lp) - 1)) + (mr - mq * kd1) + mq * kd1 * K;
            cb[j] = kD * ((cr >> lp) << lp);
        } else {
            cslot[j] = -1;
            ca[j] = 0;
            cb[j] = 0;
        }
    }
    for (int row = tid; row < m; row += kMFThreads) {
        // row block rb of level l: cell cd0 of the level, mode i along d
        const int rb = row / K, i = row - rb * K;
        const int l = block_level(rb);
        const int cd0 = l >= 2 ? rb - (1 << (l - 2)) : 0;
        rinfo[row] = make_int2((int)C.blockoff[it.boff + l - 1] + kD * (cd0 << lp) + i * kd1, l > 2 ? l - 2 : 0);
    }
    // an input written by the previous phase of this launch must be complete;
    // in a whole-step launch, so must the previous stage's RK update of the
    // stage input
    if (tid == 0) {
        if (it.win_ctr > 0) wait_counter(ctr + it.win_ctr, it.win_need, err);
        if ((it.flags & TILE_WAIT_IN) && it.wait_ctr >= 0) wait_counter(ctr + it.wait_ctr, it.wait_need, err);
    }
    __syncthreads();
    const float* __restrict__ uin = C.u[in_sel];
    if (it.src < 0) {
        // gather the stage input into X.  The copies go through L1: the input
        // was written by the previous launch or, in a whole-step launch, by
        // the previous stage's RK update of this group (which the item waited
        // for), and no L1 line can hold an older copy -- a stage-input buffer
        // is read by one stage of a launch only, after it was written, and
        // groups start on 128-byte boundaries of the buffers.
        tile_columns(W, lw, [&](int j, int r0, int rstep) {
            float* xc = X + j;
            const int s = cslot[j];
            if (s < 0) {
                for (int row = r0; row < m; row += rstep) xc[row * W] = 0.f;
                return;
            }
            const float* base = uin + (size_t)s * C.Ns + ca[j];
            const int bj = cb[j];
            for (int row = r0; row < m; row += rstep) {
                const int2 ri = rinfo[row];
                const int o = ri.x + (bj << ri.y);
                if (SGDG_IN(ca[j] + o, C.N))
                    cp_async4(xc + row * W, base + o);
                else
                    xc[row * W] = 0.f;
            }
        });
        cp_async_wait_all();
    } else {
        // a scratch vector written in this launch by other SMs: L2 loads (.cg)
        const float* __restrict__ vin = C.vbase + (size_t)it.src * C.vstride;
        const int nsum = (it.flags & TILE_SUMIN) ? C.D : 1;
        tile_columns(W, lw, [&](int j, int r0, int rstep) {
            float* xc = X + j;
            const int s = cslot[j];
            if (s < 0) {
                for (int row = r0; row < m; row += rstep) xc[row * W] = 0.f;
                return;
            }
            const float* base = vin + (size_t)s * C.N + ca[j];
            const int bj = cb[j];
            const size_t step2 = 2 * (size_t)C.vstride;
            // kOutRows rows' loads in flight at a time
            for (int row0 = r0; row0 < m; row0 += kOutRows * rstep) {
                float v[kOutRows];
#pragma unroll
                for (int u = 0; u < kOutRows; u++) {
                    const int row = row0 + u * rstep;
                    v[u] = 0.f;
                    if (row < m) {
                        const int2 ri = rinfo[row];
                        const int o = ri.x + (bj << ri.y);
                        if (SGDG_IN(ca[j] + o, C.N)) {
                            const float* p = base + o;
                            v[u] = __ldcg(p);
                            for (int q = 1; q < nsum; q++) v[u] += __ldcg(p + q * step2);  // the D products, in order
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < kOutRows; u++)
                    if (row0 + u * rstep < m) xc[(row0 + u * rstep) * W] = v[u];
            }
        });
    }
    __syncthreads();
    const int lwq = lw - (CPT == 4 ? 2 : 1);
    const int rlong = it.rlong;  // row blocks of levels <= lmax - coop (tile shape)
    auto store = [&](float* dst, int rb, int jq, float(&o)[K][CPT]) {
#pragma unroll
        for (int i = 0; i < K; i++) {
            float* yp = dst + (rb * K + i) * W + jq * CPT;
            if constexpr (CPT == 4)
                *reinterpret_cast<float4*>(yp) = make_float4(o[i][0], o[i][1], o[i][2], o[i][3]);
            else
                *reinterpret_cast<float2*>(yp) = make_float2(o[i][0], o[i][1]);
        }
    };
    // result Z of the tile: X -> Y, or for the wave's D_d D_d without the
    // squared table X -> Y -> X (X is dead after the first sweep)
    float* Z = Y;
    if (TWICE) {
        apply_rows<K, CPT>(T, X, W, nrb, lwq, rlong, [&](int rb, int jq, float(&o)[K][CPT]) { store(Y, rb, jq, o); });
        __syncthreads();
        Z = X;
    }
    apply_rows<K, CPT>(T, TWICE ? Y : X, W, nrb, lwq, rlong, [&](int rb, int jq, float(&o)[K][CPT]) { store(Z, rb, jq, o); });
    // the partial sums of this group's previous pass must be complete
    if (!(it.flags & TILE_WAIT_IN) && it.wait_ctr >= 0 && tid == 0) wait_counter(ctr + it.wait_ctr, it.wait_need, err);
    __syncthreads();
    // claim the CTA's next item now (after every wait of this one): the
    // atomic's round trip overlaps the output
    int nxt = 0;
    if (tid == 32) nxt = atomicAdd(ctr, 1);
    const bool first = (it.flags & TILE_FIRST) != 0;
    // The output loops take kOutRows rows of a column at a time and issue all
    // their loads before any store: a store may alias a later row's load as far
    // as the compiler can tell, so a row-at-a-time loop is one global round
    // trip per row.  Rows past the end load a copy of the last row (in bounds)
    // and store nothing.
    if (it.flags & (TILE_STORE | TILE_WACC)) {
        // Vlasov: a transform's result to a scratch vector, or the point
        // product w_d .* result added into the point-basis accumulator
        float* __restrict__ out = C.vbase + (size_t)it.dst * C.vstride;
        const bool wacc = (it.flags & TILE_WACC) != 0;
        tile_columns(W, lw, [&](int j, int r0, int rstep) {
            const int s = cslot[j];
            if (s < 0) return;
            float* oc = out + (size_t)s * C.N + ca[j];
            const float* wc = C.vw + (size_t)s * 2 * C.D * C.N + (size_t)it.wsel * C.N + ca[j];
            const size_t wlo = (size_t)C.D * C.N;
            const int bj = cb[j];
            for (int row0 = r0; row0 < m; row0 += kOutRows * rstep) {
                int off[kOutRows];
                bool bad[kOutRows];
                float v[kOutRows], wh[kOutRows], wl[kOutRows], prev[kOutRows];
#pragma unroll
                for (int u = 0; u < kOutRows; u++) {
                    const int row = min(row0 + u * rstep, m - 1);
                    const int2 ri = rinfo[row];
                    off[u] = ri.x + (bj << ri.y);
                    bad[u] = !SGDG_IN(ca[j] + off[u], C.N);
                    if (bad[u]) off[u] = -ca[j];  // loads the slot's first element, stores nothing
                    v[u] = Z[row * W + j];
                    wh[u] = wacc ? __ldg(wc + off[u]) : 0.f;
                    wl[u] = wacc ? __ldg(wc + wlo + off[u]) : 0.f;
                    prev[u] = wacc && !first ? __ldcg(oc + off[u]) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < kOutRows; u++) {
                    if (row0 + u * rstep >= m) break;
                    if (bad[u]) continue;
                    float x = v[u];
                    if (wacc) {
                        x = fmaf(wh[u], x, wl[u] * x);
                        if (!first) x += prev[u];
                    }
                    __stcg(oc + off[u], x);
                }
            }
        });
    } else if (!(it.flags & TILE_RK)) {
        // partial sum sum_{q <= d} coef_q D_q u of this tile's elements
        tile_columns(W, lw, [&](int j, int r0, int rstep) {
            const int s = cslot[j];
            if (s < 0) return;
            float* rc = C.rhs + (size_t)s * C.N + ca[j];
            const float chi = __ldg(C.coef + s * 16 + it.d), clo = __ldg(C.coef + s * 16 + 8 + it.d);
            const int bj = cb[j];
            for (int row0 = r0; row0 < m; row0 += kOutRows * rstep) {
                int off[kOutRows];
                bool bad[kOutRows];
                float z[kOutRows], prev[kOutRows];
#pragma unroll
                for (int u = 0; u < kOutRows; u++) {
                    const int row = min(row0 + u * rstep, m - 1);
                    const int2 ri = rinfo[row];
                    off[u] = ri.x + (bj << ri.y);
                    bad[u] = !SGDG_IN(ca[j] + off[u], C.N);
                    if (bad[u]) off[u] = -ca[j];  // loads the slot's first element, stores nothing
                    z[u] = Z[row * W + j];
                    prev[u] = first ? 0.f : __ldcg(rc + off[u]);
                }
#pragma unroll
                for (int u = 0; u < kOutRows; u++) {
                    if (row0 + u * rstep >= m) break;
                    if (bad[u]) continue;
                    float v = fmaf(chi, z[u], clo * z[u]);
                    if (!first) v += prev[u];
                    __stcg(rc + off[u], v);
                }
            }
        });
    } else {
    // last dimension: the right-hand side of each element is complete here, so
    // the RK4 stage update of its state runs in place (for the wave also the
    // element's f component, whose derivative is the stage input of v).  The
    // pencils of one dimension partition the coefficients, so every state
    // element is updated once per stage.  The FP64 state is read and written
    // once per stage: its accesses are evict-first, leaving L2 to the groups'
    // partial sums and stage inputs.
    float* __restrict__ uout = C.u[(in_sel + 1) & 3];
    constexpr int R_ = WAVE ? 2 : kOutRows;  // the wave carries two components per row
    // the stage is a compile-time constant of the element loop (one loop per
    // stage), so the RK4 formulas, the accumulator load and the stored
    // vector are fixed per loop instead of decided per element
    auto rk_loop = [&](auto stage_c) {
    constexpr int STG = decltype(stage_c)::value;
    tile_columns(W, lw, [&](int j, int r0, int rstep) {
        const int s = cslot[j];
        if (s < 0 || __ldg(C.status + s) != 0) return;
        const size_t b = (size_t)s * C.Ns + ca[j];         // the column's f component (wave) or state
        const size_t bv = b + (WAVE ? (size_t)C.N : 0);    // the component D acts on
        const float* rc = C.rhs + (size_t)s * C.N + ca[j];
        const float chi = __ldg(C.coef + s * 16 + it.d), clo = __ldg(C.coef + s * 16 + 8 + it.d);
        const double dt = __ldg(C.dt + 3 * s), hdt = __ldg(C.dt + 3 * s + 1), dt6 = __ldg(C.dt + 3 * s + 2);
        const int bj = cb[j];
        for (int row0 = r0; row0 < m; row0 += R_ * rstep) {
            int off[R_];
            bool bad[R_];
            float z[R_], prev[R_], kf[R_];
            double yv[R_], av[R_], yf[R_], af[R_];
#pragma unroll
            for (int u = 0; u < R_; u++) {
                const int row = min(row0 + u * rstep, m - 1);
                const int2 ri = rinfo[row];
                off[u] = ri.x + (bj << ri.y);
                bad[u] = !SGDG_IN(ca[j] + off[u], C.N);
                if (bad[u]) off[u] = -ca[j];  // loads the slot's first element, stores nothing
                z[u] = Z[row * W + j];
            }
#pragma unroll
            for (int u = 0; u < R_; u++) {
                prev[u] = first ? 0.f : __ldcg(rc + off[u]);
                yv[u] = ld_state(C.y + bv + off[u], pol);
                av[u] = STG != 1 ? ld_state(C.acc + bv + off[u], pol) : 0.0;
                if (WAVE) {
                    yf[u] = ld_state(C.y + b + off[u], pol);
                    af[u] = STG != 1 ? ld_state(C.acc + b + off[u], pol) : 0.0;
                    kf[u] = __ldcg(uin + b + C.N + off[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < R_; u++) {
                if (row0 + u * rstep >= m) break;
                if (bad[u]) continue;
                const int o = off[u];
                float v = fmaf(chi, z[u], clo * z[u]);
                if (!first) v += prev[u];
                double un;
                rk_stage(STG, dt, hdt, dt6, f32_to_f64(v), yv[u], av[u], un);
                if (STG == 4)
                    __stcs(C.y + bv + o, yv[u]);
                else
                    __stcs(C.acc + bv + o, av[u]);
                __stcg(uout + bv + o, f64_to_f32(un));
                if (WAVE) {
                    rk_stage(STG, dt, hdt, dt6, f32_to_f64(kf[u]), yf[u], af[u], un);
                    if (STG == 4)
                        __stcs(C.y + b + o, yf[u]);
                    else
                        __stcs(C.acc + b + o, af[u]);
                    __stcg(uout + b + o, f64_to_f32(un));
                }
            }
        }
    });
    };
    switch (stage) {
        case 1: rk_loop(std::integral_constant<int, 1>{}); break;
        case 2: rk_loop(std::integral_constant<int, 2>{}); break;
        case 3: rk_loop(std::integral_constant<int, 3>{}); break;
        default: rk_loop(std::integral_constant<int, 4>{}); break;
    }
    }
    if (tid == 32) *claim = nxt;
}

__global__ void __launch_bounds__(kMFThreads, 3)
    k_mf_stage(const MFItem* __restrict__ items, int nitems, const MFClass* __restrict__ classes, int* ctr, int lstage,
               int lin_sel, int* err, int table_bytes) {
    // dynamic shared memory: [1D operator table of the current class][tile]
    extern __shared__ __align__(16) float smem[];
    float* tile = smem + table_bytes / 4;
    __shared__ int s_item;
    __shared__ MFItem s_it;
    __shared__ MFClass s_cls;
    __shared__ int s_cls_id;   // class in s_cls (-1: none)
    __shared__ const int32_t* s_cached;  // the table in shared memory, by its global row pointers (null: none)
    const int tid = threadIdx.x;
    unsigned long long pol;  // L2 evict-first policy of the FP64 state streams
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    constexpr int kItemWords = sizeof(MFItem) / 4;
    constexpr int kClsWords = sizeof(MFClass) / 4;
    static_assert(kItemWords <= 32, "item fits one warp");
    if (tid == 0) {
        s_cls_id = -1;
        s_cached = nullptr;
    }
    if (tid == 32) s_item = atomicAdd(ctr, 1);
    int done = -1;  // thread 0: completion counter of the last finished item
    for (;;) {
        __syncthreads();  // every thread has finished the previous item; s_item is claimed
        // warp 1 stages the claimed item (and its class descriptor when the
        // class changes) while thread 0 publishes the previous item's completion
        if (tid >= 32 && tid < 64) {
            const int lane = tid - 32;
            const int ii = s_item;
            if (ii < nitems) {
                int word = 0;
                if (lane < kItemWords) {
                    word = reinterpret_cast<const int*>(items + ii)[lane];
                    reinterpret_cast<int*>(&s_it)[lane] = word;
                }
                const int cls = __shfl_sync(0xffffffffu, word, 0) >> 16;  // MFItem::cls (second int16)
                if (cls != s_cls_id)
                    for (int w = lane; w < kClsWords; w += 32)
                        reinterpret_cast<int*>(&s_cls)[w] = reinterpret_cast<const int*>(classes + cls)[w];
            }
        }
        if (tid == 0 && done >= 0) {
            __threadfence();
            atomicAdd(ctr + done, 1);
            done = -1;
        }
        __syncthreads();
        if (s_item >= nitems) break;
        const MFItem& it = s_it;
        const MFClass& C = s_cls;
        if (tid == 0) {
            s_cls_id = it.cls;  // read again only after the next barrier
            done = it.done_ctr;
        }
        // the item's table: the derivative table or a nodal transform (a
        // shared-memory copy when it fits the reserved space, cached across
        // items by its row pointers), or the wave's squared line operators
        // (through L1)
        OpTable T{C.s_rowptr, C.s_ent, C.s_val};
        int tn[3] = {C.s_nrow, C.s_nent, C.s_nval};
        bool tsh = C.s_shared != 0;
        if (it.tab == TABLE_SQUARE) {
            T = OpTable{C.q_rowptr + C.q_roff[it.lmax - 1], C.q_ent, C.q_val};
            tsh = false;
        } else if (it.tab != TABLE_DERIVATIVE) {
            T = OpTable{C.t_rowptr[it.tab], C.t_ent[it.tab], C.t_val[it.tab]};
            tn[0] = C.t_nrow[it.tab];
            tn[1] = C.t_nent[it.tab];
            tn[2] = C.t_nval[it.tab];
            tsh = mf_table_bytes(tn[0], tn[1], tn[2]) <= table_bytes;
        }
        if (tsh) {
            int* trow = reinterpret_cast<int*>(smem);
            int* tent = trow + tn[0];
            float* tval = smem + (((tn[0] + tn[1]) * 4 + 15) / 16) * 4;
            if (s_cached != T.rowptr) {  // copy the table (uniform branch; classes of one (k, n) share it)
                for (int i = tid; i < tn[0]; i += kMFThreads) trow[i] = T.rowptr[i];
                for (int i = tid; i < tn[1]; i += kMFThreads) tent[i] = T.ent[i];
                for (int i = tid; i < tn[2] / 4; i += kMFThreads)
                    reinterpret_cast<float4*>(tval)[i] = reinterpret_cast<const float4*>(T.val)[i];
                __syncthreads();
                if (tid == 0) s_cached = T.rowptr;
            }
            T = OpTable{trow, tent, tval};
        }
        // Vlasov sweeps once, like advection; the wave twice unless its
        // squared table is used.  An item of a whole-step list carries its
        // RK stage (stage input u[(stage - 1) % 2]).
        const int kind = C.kind != MF_KIND_WAVE ? 0 : it.tab == TABLE_SQUARE ? 1 : 2;
        const int stage = it.stage > 0 ? it.stage : lstage;
        const int in_sel = it.stage > 0 ? (it.stage - 1) & 3 : lin_sel;
        switch (C.k * 3 + kind) {
            case 3: pass_tile<1, 4, false, false>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 4: pass_tile<1, 4, true, false>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 5: pass_tile<1, 4, true, true>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 6: pass_tile<2, 4, false, false>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 7: pass_tile<2, 4, true, false>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 8: pass_tile<2, 4, true, true>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 9: pass_tile<3, 4, false, false>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 10: pass_tile<3, 4, true, false>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 11: pass_tile<3, 4, true, true>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 12: pass_tile<4, 2, false, false>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 13: pass_tile<4, 2, true, false>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 14: pass_tile<4, 2, true, true>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 15: pass_tile<5, 2, false, false>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 16: pass_tile<5, 2, true, false>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            case 17: pass_tile<5, 2, true, true>(it, C, T, stage, in_sel, tile, ctr, err, &s_item, pol); break;
            default:
                if (tid == 32) s_item = nitems;  // unreachable (k in 1..5): stop
                break;
        }
    }
}

// Self-test of the bounded wait: thread 0 waits for a counter that nothing
// increments; the wait gives up after kSpinLimit polls and raises *err.
__global__ void k_wait_selftest(const int* ctr, int need, int* err) {
    if (threadIdx.x == 0) wait_counter(ctr, need, err);
}

cudaError_t launch_wait_selftest(const int* ctr, int need, int* err, cudaStream_t st) {
    k_wait_selftest<<<1, 32, 0, st>>>(ctr, need, err);
    return cudaGetLastError();
}

// Self-test of the integer-pipe conversions against the hardware ones: for
// each x[i], f64_to_f32(x) and, for the float x rounds to and for the float
// whose bits are x's low word, f32_to_f64; a result that differs from the
// hardware conversion in any bit counts in bad[0], and bad[1] keeps the
// smallest such index.
__global__ void k_convert_selftest(const double* __restrict__ x, int64_t n, unsigned long long* bad) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = x[i];
        const float hw = __double2float_rn(v);
        bool ok = __float_as_uint(f64_to_f32(v)) == __float_as_uint(hw);
        const float g[2] = {hw, __uint_as_float((unsigned)__double2loint(v))};
        for (int q = 0; q < 2; q++)
            ok = ok && __double_as_longlong(f32_to_f64(g[q])) == __double_as_longlong((double)g[q]);
        if (!ok) {
            atomicAdd(bad, 1ull);
            atomicMin(bad + 1, (unsigned long long)i);
        }
    }
}

cudaError_t launch_convert_selftest(const double* x, int64_t n, unsigned long long* bad, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int64_t blocks = (n + 255) / 256;
    k_convert_selftest<<<(int)(blocks < 4096 ? blocks : 4096), 256, 0, st>>>(x, n, bad);
    return cudaGetLastError();
}

int mf_columns_per_thread(int k) { return k <= 3 ? 4 : 2; }

cudaError_t launch_mf_stage(const MFItem* items, int nitems, const MFClass* classes, int* ctr, int nctr, int stage,
                            int in_sel, int* err, size_t smem, int table_bytes, int grid, cudaStream_t st) {
    if (nitems <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(int) * (size_t)nctr, st);
    if (e != cudaSuccess) return e;
    k_mf_stage<<<grid, kMFThreads, smem, st>>>(items, nitems, classes, ctr, stage, in_sel, err, table_bytes);
    return cudaGetLastError();
}

// The dynamic shared-memory limit of k_mf_stage is one attribute per device
// for the whole process, and every engine (and the allocation-free entry
// point) launches with the size it planned: so the limit only ever rises,
// to the largest size any caller has asked for on that device.
SGDG_BOUNDS_READER(mf_bounds_violations)

cudaError_t mf_configure(size_t smem, int* blocks_per_sm) {
    static std::mutex mu;
    static std::map<int, size_t> limit;  // device -> attribute value set
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    {
        std::lock_guard<std::mutex> g(mu);
        size_t& cur = limit[dev];
        if (smem > cur) {
            e = cudaFuncSetAttribute(k_mf_stage, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            cur = smem;
        }
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_mf_stage, kMFThreads, smem);
}

}  // namespace sgdg
