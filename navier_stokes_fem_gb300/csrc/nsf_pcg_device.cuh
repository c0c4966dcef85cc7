// Preconditioned conjugate gradients with a multicolour incomplete-Cholesky-shaped factor M = L L^T (the
// reference's IC0Preconditioner path, include/assembly.h:33-35 and 1338-1344, and the learned factor).
//
// Rows are coloured so that neighbours never share a colour; L_ij (i != j) is non-zero only when colour(j) <
// colour(i).  M^-1 r is then two sweeps of colour phases, every row of a colour independent of the others:
//     forward,  c = 0 .. C-1:   y_i = (r_i - sum_{colour j < c} L_ij y_j) / L_ii
//     backward, c = C-1 .. 0:   z_i = (y_i - sum_{colour j > c} L_ji z_j) / L_ii
// Colour 0 of the forward sweep needs no neighbour, so it is fused into the phase that produces r; the backward
// step of the last colour is z_i = y_i / L_ii and is fused into that colour's forward phase.  A solve with C
// colours therefore spends 2C - 2 team barriers per iteration on the sweeps.  The factor's rows are stored as
// SELL-32 slices over per-colour row lists, so a colour phase streams contiguous, coalesced slices.
#pragma once
#include "nsf_device.cuh"

namespace nsf {

// this CTA's share [r0, r1) of the rows [c0, c1) of one colour block (both multiples of 32), in whole slices
__device__ __forceinline__ void team_block(int c0, int c1, const Team& t, int& r0, int& r1) {
    const int chunk = ((c1 - c0) / kSlice + t.size - 1) / t.size * kSlice;
    r0 = min(c1, c0 + t.rank * chunk);
    r1 = min(c1, r0 + chunk);
}

// values a sweep row needs besides its sum, loaded when its slice starts
template <typename TA> struct SweepRow {
    TA src;   // r_i (forward) or y_i (backward)
    TA d;     // 1 / L_ii
    TA r;     // r_i (backward: the r.z term)
};

// Accumulator of r.z: FP64 for the FP64 solver, double-float for the mixed one.
template <typename TA> struct DotAcc;
template <> struct DotAcc<double> {
    double v = 0.0;
    __device__ void add(double a, double b) { v = fma(a, b, v); }
    __device__ double block(double* smem) const { return block_sum(v, smem); }
};
template <> struct DotAcc<float> {
    float hi = 0.f, lo = 0.f;
    __device__ void add(float a, float b) { df_acc(hi, lo, a, b); }
    __device__ double block(double* smem) const { return block_sum_df(hi, lo, smem); }
};

// Colour-0 rows of the forward sweep (permuted rows [0, colourRow[1])), fused into the phase that writes r_i:
// y_i = r_i / L_ii (and, with a single colour, z_i = y_i / L_ii with its r.z term).
template <typename TA>
__device__ __forceinline__ void colour0_row(const FactorView& F, TA* w, const TA* dinv, int row, TA ri,
                                            DotAcc<TA>& rz) {
    if (row >= F.colourRow[1]) return;
    const TA d = dinv[row];
    TA y = ri * d;
    if (F.colours == 1) {
        y *= d;
        rz.add(ri, y);
    }
    w[row] = y;
}

// colour0_row with 1 / L_ii already loaded (d; only read for colour-0 rows)
template <typename TA>
__device__ __forceinline__ void colour0_store(const FactorView& F, TA* w, int row, TA ri, TA d, DotAcc<TA>& rz) {
    if (row >= F.colourRow[1]) return;
    TA y = ri * d;
    if (F.colours == 1) {
        y *= d;
        rz.add(ri, y);
    }
    w[row] = y;
}

// Forward colours 1..C-1 and backward colours C-2..0 of M^-1 r (colour 0 already done), then the grid-wide r.z.
// Each colour phase is the pipelined SELL-32 product over the colour's rows of L (or L^T).  `rz` holds this
// thread's r.z terms so far.  Returns false on a barrier timeout.
// One colour phase of a sweep: through the warp's ring when the kernel has one and the factor is narrow enough
// (FP32 factors), else the register-pipelined SELL-32 product.
// (Lean: one slice stream per warp, for the kernels that run at more CTAs per SM.  C16: the register product
// over the part's 16-bit column copy col16 / colBase, which the caller has checked exists.)
template <typename TV, typename TA, bool Lean = false, bool C16 = false, typename Gather, typename Pre, typename Epi>
__device__ __forceinline__ void sweep_rows(SellRing* ring, int maxW, const int* start, const int* col, const TV* val,
                                           int r0, int r1, Gather gather, Pre pre, Epi epi,
                                           const unsigned short* col16 = nullptr, const int* colBase = nullptr) {
    if constexpr (C16) {
        sell_rows<TV, TA, false, 1, 4, unsigned short>(start, col16, val, r0, r1, gather, pre, epi, colBase);
        return;
    }
    if constexpr (sizeof(TV) == 4) {
        if (ring && maxW <= kRingWidth) {
            sell_rows_ring<TA, false>(*ring, start, col, val, r0, r1, gather, pre, epi);
            return;
        }
    }
    sell_rows<TV, TA, false, (sizeof(TA) == 4 && !Lean) ? 2 : 1, 4>(start, col, val, r0, r1, gather, pre, epi);
}

// (cFirst = 2: colour 1 of the forward sweep, and with two colours its backward step, are already done.)
template <typename TV, typename TA, bool Lean = false, bool C16 = false>
__device__ bool precond_sweeps(Team& t, const CgArgs& a, const TA* r, TA* w, const TV* loVal, const TV* upVal,
                               const TA* dinv, DotAcc<TA>& rz, double* smem, int& where, double& rzOut,
                               SellRing* ring = nullptr, int cFirst = 1) {
    const FactorView& F = a.f;
    const int C = F.colours;
    for (int c = cFirst; c < C; ++c) {
        int r0, r1;
        team_block(F.colourRow[c], F.colourRow[c + 1], t, r0, r1);
        const bool last = c == C - 1;
        sweep_rows<TV, TA, Lean, C16>(ring, F.loMaxW, F.loStart, F.loCol, loVal, r0, r1, [&](int j) { return w[j]; },
                           [&](int i) { return SweepRow<TA>{r[i], dinv[i], TA(0)}; },
                           [&](int i, TA acc, const SweepRow<TA>& q) {
                               TA y = (q.src - acc) * q.d;
                               if (last) {   // backward step of the last colour: z_i = y_i / L_ii
                                   y *= q.d;
                                   rz.add(q.src, y);
                               }
                               w[i] = y;
                           }, F.loCol16, F.loColBase);
        if (!t.barrier(where++)) return false;
    }
    for (int c = C - 2; c >= 0; --c) {
        int r0, r1;
        team_block(F.colourRow[c], F.colourRow[c + 1], t, r0, r1);
        sweep_rows<TV, TA, Lean, C16>(ring, F.upMaxW, F.upStart, F.upCol, upVal, r0, r1, [&](int j) { return w[j]; },
                           [&](int i) { return SweepRow<TA>{w[i], dinv[i], r[i]}; },
                           [&](int i, TA acc, const SweepRow<TA>& q) {
                               const TA z = (q.src - acc) * q.d;
                               rz.add(q.r, z);
                               w[i] = z;
                           }, F.upCol16, F.upColBase);
        if (c > 0 && !t.barrier(where++)) return false;
    }
    const double part = rz.block(smem);
    if (threadIdx.x == 0) a.partials[4 * t.size + t.rank] = part;
    if (!t.barrier(where++)) return false;
    rzOut = grid_sum(a.partials + 4 * t.size, t.size, smem);
    return true;
}

// The preconditioned solve runs on the colour-permuted system: a.n is the padded size and a.b, a.x0 and a.x are
// the permuted vectors (F.bp, F.xp); the caller's vectors are F.natB / F.natX0 / F.natX.  In: (the fused
// right-hand side is built in the caller's order, then) b and x0 are gathered into permuted order; out: x is
// scattered back.  Returns false on a barrier timeout.
template <bool Wide = false>
static __device__ bool permute_in(Team& t, const CgArgs& a, double* stage, int& where) {
    const FactorView& F = a.f;
    int rb, re;
    team_rows(F.nNatural, t, rb, re);
    build_rhs<Wide>(a, rb, re, stage);
    if (a.bRowptr && !t.barrier(where++)) return false;
    const double* b = a.bRowptr ? a.bOut : F.natB;
    team_rows(a.n, t, rb, re);
    for (int i = rb + (int)threadIdx.x; i < re; i += blockDim.x) {
        const int o = F.perm[i];
        F.bp[i] = o >= 0 ? b[o] : 0.0;
        F.xp[i] = o >= 0 ? F.natX0[o] : 0.0;
    }
    return t.barrier(where++);
}

static __device__ void permute_out(Team& t, const CgArgs& a) {
    const FactorView& F = a.f;
    int rb, re;
    team_rows(a.n, t, rb, re);
    for (int i = rb + (int)threadIdx.x; i < re; i += blockDim.x) {
        const int o = F.perm[i];
        if (o >= 0) F.natX[o] = F.xp[i];
    }
}

// ---------------------------------------------------------------------------------------------------
// FP64 PCG.  partial regions: 0 = p.q, 1 = r.r, 2 = r0.r0, 3 = b.b, 4 = r.z
// ---------------------------------------------------------------------------------------------------
template <bool Wide = false>
static __device__ int pcg_fp64_body(Team& t, const CgArgs& a, double* stage, double* smem) {
    const FactorView& F = a.f;
    const int G = t.size, bs = blockDim.x;
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double* b = a.b;   // permuted right-hand side (permute_in)
    double* w = F.w;
    int where = 200;

    double rrp = 0, bbp = 0;
    DotAcc<double> rz0;
    matrix_product<double, double, false, kResidU<Wide>, Wide>(a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col, a.val, rb, re, stage,
                                          [&](int c) { return a.x0[c]; },
                              [&](int row, double acc, double x0i) {
                                  const double bi = b[row];
                                  const double ri = bi - acc;
                                  a.r[row] = ri;
                                  if (a.x != a.x0) a.x[row] = x0i;
                                  rrp = fma(ri, ri, rrp);
                                  bbp = fma(bi, bi, bbp);
                                  colour0_row<double>(F, w, F.dinv, row, ri, rz0);
                              });
    rrp = block_sum(rrp, smem);
    bbp = block_sum(bbp, smem);
    if (threadIdx.x == 0) { a.partials[2 * G + t.rank] = rrp; a.partials[3 * G + t.rank] = bbp; }
    if (!t.barrier(where++)) { write_info(t, a, 0, NSF_ERR_BARRIER_TIMEOUT, 1, 0, 0); return NSF_ERR_BARRIER_TIMEOUT; }
    double rr = grid_sum(a.partials + 2 * G, G, smem);
    const double bb = grid_sum(a.partials + 3 * G, G, smem);
    const double target = bb > 0 ? a.tol2 * bb : a.tol2 * rr;
    int it = 0, status = NSF_ERR_NOT_CONVERGED;
    if (!(rr == rr) || !(bb == bb) || isinf(rr) || isinf(bb)) status = NSF_ERR_BREAKDOWN;
    else if (rr <= target) status = NSF_OK;
    double rz = 0, beta = 0;
    if (status == NSF_ERR_NOT_CONVERGED) {
        if (!precond_sweeps<double, double>(t, a, a.r, w, F.loVal, F.upVal, F.dinv, rz0, smem, where, rz)) {
            write_info(t, a, 0, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb);
            return NSF_ERR_BARRIER_TIMEOUT;
        }
        if (!(rz > 0.0) || isinf(rz)) status = NSF_ERR_BREAKDOWN;
    }
    double* p = a.pbuf0;
    while (status == NSF_ERR_NOT_CONVERGED && it < a.maxIt) {
        // p = z + beta p
        for (int i0 = rb + (int)threadIdx.x; i0 < re; i0 += kRows * bs) {
            double pi[kRows], wi[kRows];
#pragma unroll
            for (int u = 0; u < kRows; ++u) {
                const int i = i0 + u * bs;
                if (i < re) {
                    pi[u] = beta == 0.0 ? 0.0 : p[i];
                    wi[u] = w[i];
                }
            }
#pragma unroll
            for (int u = 0; u < kRows; ++u) {
                const int i = i0 + u * bs;
                if (i < re) p[i] = beta == 0.0 ? wi[u] : fma(beta, pi[u], wi[u]);
            }
        }
        if (!t.barrier(where++)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb); return NSF_ERR_BARRIER_TIMEOUT; }
        // q = A p, p.q
        double pq = 0;
        matrix_product<double, double, false, kUnroll, Wide>(a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col, a.val, rb, re, stage,
                                              [&](int c) { return p[c]; },
                                              [&](int row, double acc, double pr) {
                                                  a.q[row] = acc;
                                                  pq = fma(pr, acc, pq);
                                              });
        pq = block_sum(pq, smem);
        if (threadIdx.x == 0) a.partials[t.rank] = pq;
        if (!t.barrier(where++)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb); return NSF_ERR_BARRIER_TIMEOUT; }
        const double pqs = grid_sum(a.partials, G, smem);
        if (!(pqs > 0.0) || isinf(pqs)) { status = NSF_ERR_BREAKDOWN; break; }
        const double alpha = block_scalar(smem, [&] { return rz / pqs; });
        // x += alpha p, r -= alpha q, r.r, colour-0 rows of the forward sweep
        double rrn = 0;
        DotAcc<double> rzp;
        for (int i0 = rb + (int)threadIdx.x; i0 < re; i0 += kRows * bs) {   // kRows rows' loads in flight
            double pi[kRows], qi[kRows], xi[kRows], ri[kRows], di[kRows];
#pragma unroll
            for (int u = 0; u < kRows; ++u) {
                const int i = i0 + u * bs;
                if (i < re) {
                    pi[u] = p[i];
                    qi[u] = a.q[i];
                    xi[u] = a.x[i];
                    ri[u] = a.r[i];
                    di[u] = i < F.colourRow[1] ? F.dinv[i] : 0.0;
                }
            }
#pragma unroll
            for (int u = 0; u < kRows; ++u) {
                const int i = i0 + u * bs;
                if (i < re) {
                    a.x[i] = fma(alpha, pi[u], xi[u]);
                    const double rn = fma(-alpha, qi[u], ri[u]);
                    a.r[i] = rn;
                    rrn = fma(rn, rn, rrn);
                    colour0_store<double>(F, w, i, rn, di[u], rzp);
                }
            }
        }
        rrn = block_sum(rrn, smem);
        if (threadIdx.x == 0) a.partials[G + t.rank] = rrn;
        if (!t.barrier(where++)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb); return NSF_ERR_BARRIER_TIMEOUT; }
        rr = grid_sum(a.partials + G, G, smem);
        ++it;
        if (!(rr == rr) || isinf(rr)) { status = NSF_ERR_BREAKDOWN; break; }
        if (rr <= target) { status = NSF_OK; break; }
        double rzn = 0;
        if (!precond_sweeps<double, double>(t, a, a.r, w, F.loVal, F.upVal, F.dinv, rzp, smem, where, rzn)) {
            write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb);
            return NSF_ERR_BARRIER_TIMEOUT;
        }
        if (!(rzn > 0.0) || isinf(rzn)) { status = NSF_ERR_BREAKDOWN; break; }
        beta = block_scalar(smem, [&] { return rzn / rz; });
        rz = rzn;
    }
    if (status == NSF_ERR_NOT_CONVERGED && a.fallbackMaxIt > 0) {
        // over the cap: plain FP64 CG from the current iterate (x is complete after the last barrier)
        CgArgs f = a;
        f.bRowptr = nullptr;
        f.b = b;
        f.x0 = a.x;
        f.maxIt = a.fallbackMaxIt;
        const int fst = team_cg_fp64<Wide>(t, f, stage, smem);
        if (fst == NSF_ERR_BARRIER_TIMEOUT) return fst;
        if (t.rank == 0 && threadIdx.x == 0) {
            a.info->iterations += it;
            a.info->fallback = 1;
        }
        return fst;
    }
    write_info(t, a, it, status, 1, rr, bb);
    return status;
}

// ---------------------------------------------------------------------------------------------------
// Mixed-precision PCG: the mixed CG of nsf_device.cuh (FP32 matrix, vectors and factor; FP64 dots, scalars,
// true residuals) with z = M^-1 r applied in FP32 after every update of r.  The search direction is formed on the
// fly in the product, p_j = z_j + beta p_prev_j.  If the recurrence stalls, or the preconditioned method needs
// more iterations than the caller allows (the plain method's count), the solve finishes with plain FP64 CG.
// partial regions: 0 = p.q, 1 = r32.r32, 2 = r64.r64, 3 = b.b, 4 = r.z
// ---------------------------------------------------------------------------------------------------
// Mixed-precision PCG on the permuted system, as two steps over a PcgLoop state:
//   refresh: (fold the FP32 correction into x,) true residual b - A64 x in FP64, the stopping and stagnation tests,
//            the sweeps of M^-1 r, and the restart decision for the recurrence;
//   inner:   FP32 iterations (product, x/r update, sweeps) until the FP32 residual has fallen by innerTol since the
//            last true residual, the stopping test is met or the iteration budget is spent.
// Both return false on a barrier time-out.  partial regions: 0 = p.q, 1 = r.r, 2 = r64.r64, 3 = b.b, 4 = r.z
__device__ __forceinline__ void pcg_loop_init(PcgLoop& L) {
    L.rr64 = L.bb = L.target = L.rz = L.beta = 0.0;
    L.scale = 1.0;
    L.rrBest = L.rrCycle = INFINITY;
    L.rrRef = 0.0;
    L.it = L.refresh = L.stalls = L.itRef = 0;
    L.first = 1;
    L.resetP = 1;
    L.flip = 0;
    L.innerBreakdown = 0;
    L.rflip = 0;
    L.state = kLoopRefresh;
    L.status = NSF_ERR_NOT_CONVERGED;
}

template <bool Wide = false>
static __device__ bool pcg_mixed_refresh(Team& t, const CgArgs& a, double* stage, double* smem, SellRing* ring,
                                         PcgLoop& L, int& where) {
    const FactorView& F = a.f;
    const int G = t.size, bs = blockDim.x;
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double* b = a.b;   // permuted right-hand side (permute_in); x0 == x
    float* w = F.w32;
    float* pprev = L.flip ? a.p32b : a.p32a;
    float* r32 = L.rflip ? a.r32b : a.r32;   // the current residual buffer
    const double sc = L.scale;                // (the power-of-two scaling of team_cg_mixed's refresh)
    if (!L.first) {   // fold the FP32 correction into x; the true residual gathers x across blocks
        const double inv = 1.0 / sc;
        for (int i = rb + (int)threadIdx.x; i < re; i += bs) a.x[i] += (double)a.d32[i] * inv;
        if (!t.barrier(where++)) return false;
        if (L.innerBreakdown) L.resetP = 1;
    }
    // true residual r = b - A64 x, r32 = (float) (scale r), d32 = 0, colour 0 of the forward sweep
    const double* xs = L.first ? a.x0 : a.x;
    const bool resetP = L.resetP != 0;
    double rrp = 0, bbp = 0;
    DotAcc<float> rzp;
    matrix_product<double, double, false, kResidU<Wide>, Wide>(a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col, a.val, rb, re,
                                                   stage, [&](int c) { return xs[c]; },
                                                   [&](int row, double acc, double) {
                                                       const double bi = b[row];
                                                       const double ri = bi - acc;
                                                       const float rf = (float)(ri * sc);
                                                       r32[row] = rf;
                                                       a.d32[row] = 0.0f;
                                                       if (resetP) pprev[row] = 0.0f;   // restart: p = z
                                                       rrp = fma(ri, ri, rrp);
                                                       bbp = fma(bi, bi, bbp);
                                                       colour0_row<float>(F, w, F.dinv32, row, rf, rzp);
                                                   });
    rrp = block_sum(rrp, smem);
    bbp = block_sum(bbp, smem);
    if (threadIdx.x == 0) {
        a.partials[2 * G + t.rank] = rrp;
        a.partials[3 * G + t.rank] = bbp;
    }
    if (!t.barrier(where++)) return false;
    L.rr64 = grid_sum(a.partials + 2 * G, G, smem);
    if (L.first) {
        L.bb = grid_sum(a.partials + 3 * G, G, smem);
        L.target = L.bb > 0 ? a.tol2 * L.bb : a.tol2 * L.rr64;
    }
    L.state = kLoopDone;
    if (!(L.rr64 == L.rr64) || isinf(L.rr64)) { L.status = NSF_ERR_BREAKDOWN; return true; }
    if (L.rr64 <= L.target) { L.status = NSF_OK; return true; }
    if (L.it >= a.maxIt || L.refresh >= a.maxOuter) return true;
    if (L.refresh > 0 && L.rr64 > 0.81 * L.rrBest) {   // stagnation guard (see team_cg_mixed)
        if (++L.stalls >= 3) return true;
    } else {
        L.stalls = 0;
    }
    L.rrBest = fmin(L.rrBest, L.rr64);
    const double f = rescale_factor(L.rr64 * sc * sc / a.n);
    if (f != 1.0) {   // own rows of r32, of y0 (colour 0) and of the previous direction; gathered after a barrier
        const float ff = (float)f;
        for (int i = rb + (int)threadIdx.x; i < re; i += bs) {
            r32[i] *= ff;
            pprev[i] *= ff;
            if (i < F.colourRow[1]) w[i] *= ff;
        }
        rzp.hi *= ff * ff;
        rzp.lo *= ff * ff;
        L.rz *= f * f;   // the previous cycle's r.z, for beta
        L.scale = sc * f;
        if (!t.barrier(where++)) return false;
    }
    double rzT = 0;
    if (!precond_sweeps<float, float>(t, a, r32, w, F.loVal32, F.upVal32, F.dinv32, rzp, smem, where, rzT, ring))
        return false;
    if (!(rzT > 0.0) || isinf(rzT)) { L.status = NSF_ERR_BREAKDOWN; return true; }
    // Continue the recurrence from the refreshed residual (beta' = r.z / r_prev.z_prev), unless the cycle just
    // ended has drifted: its FP32 recursive residual fell by innerTol^2 but the true one by less than a quarter.
    // Then restart it (p = z).  Carried recurrences converged fastest on the large pressure systems once the flow
    // had settled, but in the first steps of a cavity they drifted and took up to 5x the iterations.
    const bool drifted = L.refresh > 0 && L.rr64 > 0.25 * L.rrCycle;
    L.beta = (L.resetP || drifted) ? 0.0 : rzT / L.rz;
    L.resetP = 0;
    L.rz = rzT;
    L.rrCycle = L.rr64;
    L.rrRef = L.rr64;
    L.itRef = L.it;
    ++L.refresh;
    L.first = 0;
    L.state = kLoopInner;
    return true;
}

template <bool Wide = false, bool Lean = false>
static __device__ bool pcg_mixed_inner(Team& t, const CgArgs& a, double* stage, double* smem, SellRing* ring,
                                       PcgLoop& L, int& where) {
    const FactorView& F = a.f;
    const int G = t.size, bs = blockDim.x;
    int rb, re;
    team_rows(a.n, t, rb, re);
    float* w = F.w32;
    L.innerBreakdown = 0;
    const double rrStop = fmax(a.innerTol2 * L.rrRef, L.target) * L.scale * L.scale;   // in the FP32 vectors' scale
    const double invScale = 1.0 / L.scale;
    while (L.it < a.maxIt) {
        const float betaf = (float)L.beta;
        const float* pp = L.flip ? a.p32b : a.p32a;
        float* pc = L.flip ? a.p32a : a.p32b;
        float pqHi = 0.f, pqLo = 0.f;
        product32<Wide, Lean ? 6 : kUnroll>(ring, a, rb, re, reinterpret_cast<float*>(stage),
                        [&](int c) { return fmaf(betaf, pp[c], w[c]); },
                        [&](int row, float acc, float pi) {
                            pc[row] = pi;
                            a.q32[row] = acc;
                            df_acc(pqHi, pqLo, pi, acc);
                        });
        const double pq = block_sum_df(pqHi, pqLo, smem);
        if (threadIdx.x == 0) a.partials[t.rank] = pq;
        if (!t.barrier(where++)) return false;
        const double pqs = grid_sum(a.partials, G, smem);
        if (!(pqs > 0.0) || isinf(pqs)) { L.innerBreakdown = 1; break; }
        const float alphaf = (float)block_scalar(smem, [&] { return L.rz / pqs; });
        const bool fold = fold_iteration(L);
        float rrHi = 0.f, rrLo = 0.f;
        DotAcc<float> rzn;
        constexpr int R = Lean ? kRowsLean : kRows;
        for (int i0 = rb + (int)threadIdx.x; i0 < re; i0 += R * bs) {   // R rows' loads in flight
            float pi[R], qi[R], di[R], ri[R], vi[R];
#pragma unroll
            for (int u = 0; u < R; ++u) {
                const int i = i0 + u * bs;
                if (i < re) {
                    pi[u] = pc[i];
                    qi[u] = a.q32[i];
                    di[u] = a.d32[i];
                    ri[u] = a.r32[i];
                    vi[u] = i < F.colourRow[1] ? F.dinv32[i] : 0.0f;
                }
            }
#pragma unroll
            for (int u = 0; u < R; ++u) {
                const int i = i0 + u * bs;
                if (i < re) {
                    a.d32[i] = fold_correction(a, i, fmaf(alphaf, pi[u], di[u]), fold, invScale);
                    const float rn = fmaf(-alphaf, qi[u], ri[u]);
                    a.r32[i] = rn;
                    df_acc(rrHi, rrLo, rn, rn);
                    colour0_store<float>(F, w, i, rn, vi[u], rzn);
                }
            }
        }
        const double rrn = block_sum_df(rrHi, rrLo, smem);
        if (threadIdx.x == 0) a.partials[G + t.rank] = rrn;
        if (!t.barrier(where++)) return false;
        const double rrs = grid_sum(a.partials + G, G, smem);
        ++L.it;
        L.flip ^= 1;
        if (!(rrs == rrs) || isinf(rrs)) { L.innerBreakdown = 1; break; }
        if (rrs <= rrStop) break;   // time for a true residual
        if (L.it - L.itRef >= kMaxInnerBetweenRefresh) break;
        double rzs = 0;
        if (!precond_sweeps<float, float, Lean>(t, a, a.r32, w, F.loVal32, F.upVal32, F.dinv32, rzn, smem, where, rzs, ring))
            return false;
        if (!(rzs > 0.0) || isinf(rzs)) { L.innerBreakdown = 1; break; }
        L.beta = block_scalar(smem, [&] { return rzs / L.rz; });
        L.rz = rzs;
    }
    L.state = kLoopRefresh;
    return true;
}

// The split form's inner iterations with the x/r update fused into colour 1 of the forward sweep (two or more
// colours): colour-0 rows update d, r and y0 = r0 / L_00 as before; colour-1 rows update their d and r in the
// sweep's pre step and take their lower neighbours' y0 from the previous residual, y0_j = (r_j - alpha q_j) / L_jj
// (the same arithmetic as the stored y0, so the sweep sees the same values); rows of colours >= 2 update d and r.  The residual alternates between two buffers, since the neighbours' previous r is read while the
// own rows' new r is written.  On two colours an iteration has 3 grid barriers instead of 4.
// (C16: the product and the sweeps read the 16-bit column copies of the matrix and of both factor parts.)
//
// Resident (two colours only, one CTA per SM): the rows a CTA updates are the same in every phase - its share of
// each colour block, the product included - so the state only that CTA reads lives in its shared memory `rs` for
// the whole launch instead of in HBM: the FP32 correction d of all its rows, and r and q of its colour-1 rows
// (no other CTA gathers them: the colour-1 sweep gathers colour-0 neighbours only, and with two colours the
// backward sweep is colour 0's).  Layout in nsf_row_state: d of the colour-0 rows, d of the colour-1 rows, r1, q1.  d and r1 are
// loaded when the launch starts and written back when it ends; 16 of the about 118 bytes per row and iteration
// that the iterations move stay on the chip.
extern __shared__ __align__(16) float nsf_row_state[];   // the resident form's dynamic shared memory

// (H16: the factor's FP16 value copies, with C16.)
template <bool C16 = false, bool Resident = false, bool H16 = false>
static __device__ bool pcg_mixed_inner_fused(Team& t, const CgArgs& a, double* stage, double* smem, SellRing* ring,
                                             PcgLoop& L, int& where) {
    using TF = std::conditional_t<H16, __half, float>;   // the factor values the sweeps read
    const TF* loV;
    const TF* upV;
    if constexpr (H16) {
        loV = a.f.loVal16;
        upV = a.f.upVal16;
    } else {
        loV = a.f.loVal32;
        upV = a.f.upVal32;
    }
    const FactorView& F = a.f;
    const int G = t.size, bs = blockDim.x, C = F.colours;
    int rb, re;
    team_rows(a.n, t, rb, re);
    float* w = F.w32;
    const float* dinv = F.dinv32;
    L.innerBreakdown = 0;
    // Resident: this CTA's colour-0 rows [c0b, c0b + n0) and colour-1 rows [c1b, c1b + n1); their state is indexed
    // in the kernel's dynamic shared memory (nsf_row_state) by 32-bit offsets: d0 at [0, n0), d1 at [n0, n0 + n1),
    // r1 at n0 + n1, q1 at n0 + 2 n1
    int c0b = 0, c1b = 0, n0 = 0, n1 = 0;
    if constexpr (Resident) {
        int e0, e1;
        team_block(F.colourRow[0], F.colourRow[1], t, c0b, e0);
        team_block(F.colourRow[1], F.colourRow[2], t, c1b, e1);
        n0 = e0 - c0b;
        n1 = e1 - c1b;
        const float* rCur = L.rflip ? a.r32b : a.r32;
        for (int k = threadIdx.x; k < n0; k += bs) nsf_row_state[k] = a.d32[c0b + k];
        for (int k = threadIdx.x; k < n1; k += bs) {
            nsf_row_state[n0 + k] = a.d32[c1b + k];
            nsf_row_state[n0 + n1 + k] = rCur[c1b + k];
        }
        __syncthreads();
    }
    // The tests on p.q and r.r and the coefficient alpha are thread 0's, handed to every thread as decisions; the
    // r.z test and beta stay per thread (thread 0 alone owning them made the 64-register kernel spill).
    const double rrStop = fmax(a.innerTol2 * L.rrRef, L.target) * L.scale * L.scale;   // in the FP32 vectors' scale
    const double invScale = 1.0 / L.scale;
    float betaf = (float)L.beta;
    while (L.it < a.maxIt) {
        const float* pp = L.flip ? a.p32b : a.p32a;
        float* pc = L.flip ? a.p32a : a.p32b;
        const float* rOld = L.rflip ? a.r32b : a.r32;
        float* rNew = L.rflip ? a.r32 : a.r32b;
        float pqHi = 0.f, pqLo = 0.f;
        auto gp = [&](int c) { return fmaf(betaf, pp[c], w[c]); };
        auto ep = [&](int row, float acc, float pi) {
            pc[row] = pi;
            a.q32[row] = acc;
            df_acc(pqHi, pqLo, pi, acc);
        };
        // chunks as wide as the widest slice when that is 5 (a structured P1 system without its exact zeros)
        if constexpr (Resident) {
            // this CTA's colour-0 share, then its colour-1 share, whose q stays in shared memory
            auto ep1 = [&](int row, float acc, float pi) {
                pc[row] = pi;
                nsf_row_state[n0 + 2 * n1 + row - c1b] = acc;
                df_acc(pqHi, pqLo, pi, acc);
            };
            if (a.sellMaxW <= 5) {
                product32<false, 5, C16>(ring, a, c0b, c0b + n0, reinterpret_cast<float*>(stage), gp, ep);
                product32<false, 5, C16>(ring, a, c1b, c1b + n1, reinterpret_cast<float*>(stage), gp, ep1);
            } else {
                product32<false, 6, C16>(ring, a, c0b, c0b + n0, reinterpret_cast<float*>(stage), gp, ep);
                product32<false, 6, C16>(ring, a, c1b, c1b + n1, reinterpret_cast<float*>(stage), gp, ep1);
            }
        } else if (a.sellMaxW <= 5) {
            product32<false, 5, C16>(ring, a, rb, re, reinterpret_cast<float*>(stage), gp, ep);
        } else {
            product32<false, 6, C16>(ring, a, rb, re, reinterpret_cast<float*>(stage), gp, ep);
        }
        const double pq = block_sum_df(pqHi, pqLo, smem);
        if (threadIdx.x == 0) a.partials[t.rank] = pq;
        if (!t.barrier(where++)) return false;
        {
            const double pqs = grid_sum0(a.partials, G);
            if (threadIdx.x == 0) {
                const bool bad = !(pqs > 0.0) || isinf(pqs);
                decision_put(smem, bad ? 0.f : (float)(L.rz / pqs), bad);
            }
        }
        const Decision da = decision_get(smem);
        if (da.code) { L.innerBreakdown = 1; break; }
        const float alphaf = da.v;
        const bool fold = fold_iteration(L);
        float rrHi = 0.f, rrLo = 0.f;
        DotAcc<float> rzn;
        // colours other than 1: d += alpha p, r -= alpha q; colour 0 also y0 = r / L_00
        for (int c = 0; c < C; ++c) {
            if (c == 1) continue;
            int r0, r1;
            team_block(F.colourRow[c], F.colourRow[c + 1], t, r0, r1);
            for (int i0 = r0 + (int)threadIdx.x; i0 < r1; i0 += kRowsLean * bs) {
                float pi[kRowsLean], qi[kRowsLean], di[kRowsLean], ri[kRowsLean], vi[kRowsLean];
#pragma unroll
                for (int u = 0; u < kRowsLean; ++u) {
                    const int i = i0 + u * bs;
                    if (i < r1) {
                        pi[u] = pc[i];
                        qi[u] = a.q32[i];
                        if constexpr (Resident) di[u] = nsf_row_state[i - c0b];   // (Resident: c == 0 only)
                        else di[u] = a.d32[i];
                        ri[u] = rOld[i];
                        vi[u] = c == 0 ? dinv[i] : 0.0f;
                    }
                }
#pragma unroll
                for (int u = 0; u < kRowsLean; ++u) {
                    const int i = i0 + u * bs;
                    if (i < r1) {
                        const float dn = fold_correction(a, i, fmaf(alphaf, pi[u], di[u]), fold, invScale);
                        if constexpr (Resident) nsf_row_state[i - c0b] = dn;
                        else a.d32[i] = dn;
                        const float rn = fmaf(-alphaf, qi[u], ri[u]);
                        rNew[i] = rn;
                        df_acc(rrHi, rrLo, rn, rn);
                        if (c == 0) w[i] = rn * vi[u];
                    }
                }
            }
        }
        // colour 1: its d and r in the pre step, y1 = (r1 - sum L_1j y0_j) / L_11 (and z1 = y1 / L_11 when it is the
        // last colour)
        {
            int r0, r1;
            team_block(F.colourRow[1], F.colourRow[2], t, r0, r1);
            const bool last = C == 2;
            using TC = std::conditional_t<C16, unsigned short, int>;
            const TC* loCol;
            if constexpr (C16) loCol = F.loCol16;
            else loCol = F.loCol;
            sell_rows<TF, float, false, 1, 4, TC>(
                F.loStart, loCol, loV, r0, r1,
                [&](int j) { return fmaf(-alphaf, a.q32[j], rOld[j]) * dinv[j]; },
                [&](int i) {
                    float rn;
                    if constexpr (Resident) {
                        const int k = i - c1b;
                        rn = fmaf(-alphaf, nsf_row_state[n0 + 2 * n1 + k], nsf_row_state[n0 + n1 + k]);
                        nsf_row_state[n0 + k] =
                            fold_correction(a, i, fmaf(alphaf, pc[i], nsf_row_state[n0 + k]), fold, invScale);
                        nsf_row_state[n0 + n1 + k] = rn;
                    } else {
                        rn = fmaf(-alphaf, a.q32[i], rOld[i]);
                        a.d32[i] = fold_correction(a, i, fmaf(alphaf, pc[i], a.d32[i]), fold, invScale);
                        rNew[i] = rn;
                    }
                    df_acc(rrHi, rrLo, rn, rn);
                    return SweepRow<float>{rn, dinv[i], 0.0f};
                },
                [&](int i, float acc, const SweepRow<float>& q) {
                    float y = (q.src - acc) * q.d;
                    if (last) {   // backward step of the last colour: z_i = y_i / L_ii
                        y *= q.d;
                        rzn.add(q.src, y);
                    }
                    w[i] = y;
                }, F.loColBase);
        }
        const double rrn = block_sum_df(rrHi, rrLo, smem);
        if (threadIdx.x == 0) a.partials[G + t.rank] = rrn;
        if (!t.barrier(where++)) return false;
        {
            const double rrs = grid_sum0(a.partials + G, G);
            if (threadIdx.x == 0) decision_put(smem, 0.f, !(rrs == rrs) || isinf(rrs) ? 1 : rrs <= rrStop ? 2 : 0);
        }
        const Decision dr = decision_get(smem);
        ++L.it;
        L.flip ^= 1;
        L.rflip ^= 1;
        if (dr.code == 1) { L.innerBreakdown = 1; break; }
        if (dr.code == 2) break;   // time for a true residual
        if (L.it - L.itRef >= kMaxInnerBetweenRefresh) break;
        double rzs = 0;
        if (!precond_sweeps<TF, float, true, C16>(t, a, rNew, w, loV, upV, dinv, rzn, smem, where,
                                                     rzs, ring, 2))
            return false;
        if (!(rzs > 0.0) || isinf(rzs)) { L.innerBreakdown = 1; break; }
        L.beta = block_scalar(smem, [&] { return rzs / L.rz; });
        L.rz = rzs;
        betaf = (float)L.beta;
    }
    if constexpr (Resident) {   // d of every own row and r of the colour-1 rows back to their global copies
        __syncthreads();
        float* rCur = L.rflip ? a.r32b : a.r32;
        for (int k = threadIdx.x; k < n0; k += bs) a.d32[c0b + k] = nsf_row_state[k];
        for (int k = threadIdx.x; k < n1; k += bs) {
            a.d32[c1b + k] = nsf_row_state[n0 + k];
            rCur[c1b + k] = nsf_row_state[n0 + n1 + k];
        }
    }
    L.state = kLoopRefresh;
    return true;
}

// ---------------------------------------------------------------------------------------------------
// Reduced (Schur complement) form of the split mixed PCG, two colours.  With two colours the colour-0 block A_00
// of the permuted matrix is diagonal, so the colour-0 unknowns can be eliminated exactly:
//     S x_1 = b_1 - A_10 A_00^-1 b_0,   S = A_11 - A_10 A_00^-1 A_01,   x_0 = A_00^-1 (b_0 - A_01 x_1).
// The iteration is PCG on S with the factor's colour-1 diagonal as preconditioner, z_1 = r_1 / L_11^2, written in
// the full system's vectors: every refresh projects x_0 (one exact Jacobi step on the colour-0 rows), so r_0 = 0;
// the search direction's colour-0 part is u_0 = -A_00^-1 A_01 p_1, which makes q_0 = (A p)_0 = 0, and
// q_1 = A_10 u_0 + A_11 p_1 = S p_1.  For IC(0) (L_00^2 = A_00, L_10 = A_10 L_00^-1, L_11^2 = diag S) these are the
// iterates of the full PCG: its z_0 = -A_00^-1 A_01 z_1 when r_0 = 0.  An iteration reads each matrix row once,
// the colour-0 rows for u_0 and the colour-1 rows for q_1, and neither factor part: about half of the full
// iteration's matrix entries and gathers, with the same three grid barriers.
//   H1, colour-0 rows:  u_i = -(1/a_ii) sum_j a_ij (z_j + beta p_j)            (stored as p_i)
//   H2, colour-1 rows:  p_i = z_i + beta p_i,  q_i = sum_j a_ij (u_j - p_i) + rowsum_i p_i,  partial p.q
//   U,  colour-1 rows:  d_i += alpha p_i,  r_i -= alpha q_i,  z_i = r_i / L_ii^2,  partials r.r and r.z
// (u_i is a weighted mean of its neighbours' p_j on a stiffness matrix, so its FP32 sum does not cancel; q_1 is
// taken in the difference form of the other mixed products.)
template <bool Wide = false>
static __device__ bool pcg_mixed_refresh_reduced(Team& t, const CgArgs& a, double* stage, double* smem, PcgLoop& L,
                                                 int& where) {
    const FactorView& F = a.f;
    const int G = t.size, bs = blockDim.x, c1 = F.colourRow[1];
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double* b = a.b;   // permuted right-hand side (permute_in); x0 == x
    double* x = a.x;
    float* w = F.w32;
    float* pprev = L.flip ? a.p32b : a.p32a;
    float* r32 = L.rflip ? a.r32b : a.r32;
    const double sc = L.scale;
    if (!L.first) {   // fold the FP32 correction into x (colour-1 rows carry one; colour-0 rows hold zero)
        const double inv = 1.0 / sc;
        for (int i = rb + (int)threadIdx.x; i < re; i += bs) a.x[i] += (double)a.d32[i] * inv;
        if (L.innerBreakdown) L.resetP = 1;
    } else if (x != a.x0) {
        for (int i = rb + (int)threadIdx.x; i < re; i += bs) x[i] = a.x0[i];
    }
    if (!t.barrier(where++)) return false;
    // x_0 = A_00^-1 (b_0 - A_01 x_1): x_i += (b_i - (A x)_i) / a_ii on the own colour-0 rows (which couple to
    // colour-1 unknowns and their own diagonal only)
    const int pe = min(re, c1);
    if (rb < pe)
        matrix_product<double, double, false, kResidU<Wide>, Wide>(
            a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col, a.val, rb, pe, stage, [&](int c) { return x[c]; },
            [&](int row, double acc, double xi) { x[row] = xi + (b[row] - acc) / F.aDiag[row]; });
    if (!t.barrier(where++)) return false;
    // true residual r = b - A64 x in FP64 (r_0 = 0 up to rounding), kept in a.r until the FP32 scale is known;
    // d32 = 0
    const bool resetP = L.resetP != 0;
    double rrp = 0, bbp = 0;
    matrix_product<double, double, false, kResidU<Wide>, Wide>(
        a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col, a.val, rb, re, stage, [&](int c) { return x[c]; },
        [&](int row, double acc, double) {
            const double bi = b[row];
            const double ri = bi - acc;
            a.r[row] = ri;
            a.d32[row] = 0.0f;
            if (resetP) pprev[row] = 0.0f;   // restart: p = z
            rrp = fma(ri, ri, rrp);
            bbp = fma(bi, bi, bbp);
        });
    rrp = block_sum(rrp, smem);
    bbp = block_sum(bbp, smem);
    if (threadIdx.x == 0) {
        a.partials[2 * G + t.rank] = rrp;
        a.partials[3 * G + t.rank] = bbp;
    }
    if (!t.barrier(where++)) return false;
    L.rr64 = grid_sum(a.partials + 2 * G, G, smem);
    if (L.first) {
        L.bb = grid_sum(a.partials + 3 * G, G, smem);
        L.target = L.bb > 0 ? a.tol2 * L.bb : a.tol2 * L.rr64;
    }
    L.state = kLoopDone;
    if (!(L.rr64 == L.rr64) || isinf(L.rr64)) { L.status = NSF_ERR_BREAKDOWN; return true; }
    if (L.rr64 <= L.target) { L.status = NSF_OK; return true; }
    if (L.it >= a.maxIt || L.refresh >= a.maxOuter) return true;
    if (L.refresh > 0 && L.rr64 > 0.81 * L.rrBest) {   // stagnation guard (see team_cg_mixed)
        if (++L.stalls >= 3) return true;
    } else {
        L.stalls = 0;
    }
    L.rrBest = fmin(L.rrBest, L.rr64);
    // the FP32 vectors at the new scale (formed after it is known, so that a tiny residual does not underflow):
    // r32 = (float) (scale r), z_1 = r_1 / L_11^2, the previous direction rescaled
    const double f = rescale_factor(L.rr64 * sc * sc / a.n);
    const double sc2 = sc * f;
    const float ff = (float)f;
    DotAcc<float> rzp;
    for (int i = rb + (int)threadIdx.x; i < re; i += bs) {
        const float rf = (float)(a.r[i] * sc2);
        r32[i] = rf;
        if (f != 1.0) pprev[i] *= ff;
        if (i >= c1) {
            const float d = F.dinv32[i];
            const float z = (rf * d) * d;
            w[i] = z;
            rzp.add(rf, z);
        }
    }
    L.rz *= f * f;   // the previous cycle's r.z, for beta (products of powers of two are exact)
    L.scale = sc2;
    const double rzb = rzp.block(smem);
    if (threadIdx.x == 0) a.partials[4 * G + t.rank] = rzb;
    if (!t.barrier(where++)) return false;
    const double rzT = grid_sum(a.partials + 4 * G, G, smem);
    if (!(rzT > 0.0) || isinf(rzT)) { L.status = NSF_ERR_BREAKDOWN; return true; }
    const bool drifted = L.refresh > 0 && L.rr64 > 0.25 * L.rrCycle;   // (see pcg_mixed_refresh)
    L.beta = (L.resetP || drifted) ? 0.0 : rzT / L.rz;
    L.resetP = 0;
    L.rz = rzT;
    L.rrCycle = L.rr64;
    L.rrRef = L.rr64;
    L.itRef = L.it;
    ++L.refresh;
    L.first = 0;
    L.state = kLoopInner;
    return true;
}

// The inner iterations of the reduced form (H1, H2, U above); the residual is updated in place, since no phase
// gathers it.  (C16: the 16-bit column copy of the matrix, whose diagonal entries are padding.  Resident: the row
// state only the owning CTA reads - d of its colour-0 rows, and d, r and q of its colour-1 rows - lives in the
// kernel's dynamic shared memory for the whole launch: nsf_row_state holds d1 at [0, n1), r1 at [n1, 2 n1), q1 at
// [2 n1, 3 n1) and d0 at [3 n1, 3 n1 + n0); d and r are loaded when the launch starts, d is written back when it
// ends (the refresh recomputes r).)
// (Schur: q_1 = S p_1 in one phase with the explicitly formed Schur complement (FactorView::sStart ..., 16-bit
// columns, difference form with its FP64 row sums), so H1, its barrier and u_0 fall away; the colour-0 unknowns
// follow from the refresh's projection alone.)
template <bool C16 = false, bool Resident = false, bool Schur = false>
static __device__ bool pcg_mixed_inner_reduced(Team& t, const CgArgs& a, double* smem, PcgLoop& L, int& where) {
    const FactorView& F = a.f;
    const int G = t.size, bs = blockDim.x, c1 = F.colourRow[1];
    float* w = F.w32;
    const float* dinv = F.dinv32;
    const float* ainv = F.aInv32;
    float* r = L.rflip ? a.r32b : a.r32;
    int a0, a1, b0, b1;   // own colour-0 rows [a0, a1) and colour-1 rows [b0, b1)
    team_block(F.colourRow[0], F.colourRow[1], t, a0, a1);
    team_block(F.colourRow[1], F.colourRow[2], t, b0, b1);
    using TC = std::conditional_t<C16, unsigned short, int>;
    const TC* col;
    if constexpr (C16) col = a.sellCol16;
    else col = a.sellCol;
    const int n0 = a1 - a0, n1 = b1 - b0;
    float* sd1 = nsf_row_state;
    float* sr1 = nsf_row_state + n1;
    float* sq1 = nsf_row_state + 2 * n1;
    float* sd0 = nsf_row_state + 3 * n1;
    // (Schur, Resident: the colour-0 correction is not kept, and 1 / L_11 of the CTA's colour-1 rows takes its place
    // in shared memory, [3 n1, 4 n1))
    float* sv1 = nsf_row_state + 3 * n1;
    if constexpr (Resident) {
        for (int k = threadIdx.x; k < n1; k += bs) {
            sd1[k] = a.d32[b0 + k];
            sr1[k] = r[b0 + k];
            if constexpr (Schur) sv1[k] = dinv[b0 + k];
        }
        if constexpr (!Schur)
            for (int k = threadIdx.x; k < n0; k += bs) sd0[k] = a.d32[a0 + k];
        __syncthreads();
    }
    L.innerBreakdown = 0;
    const double rrStop = fmax(a.innerTol2 * L.rrRef, L.target) * L.scale * L.scale;   // in the FP32 vectors' scale
    const double invScale = 1.0 / L.scale;
    float betaf = (float)L.beta;
    while (L.it < a.maxIt) {
        const float* pp = L.flip ? a.p32b : a.p32a;
        float* pc = L.flip ? a.p32a : a.p32b;
        // H1: u_0 (the colour-0 columns of a colour-0 row are its own diagonal only: excluded)
        if constexpr (!Schur) {
        auto h1 = [&](auto U) {
            sell_rows<float, float, false, 1, decltype(U)::value, TC>(
                a.sellStart, col, a.sellVal32, a0, a1,
                [&](int j) { return j >= c1 ? fmaf(betaf, pp[j], w[j]) : 0.0f; }, [&](int i) { return ainv[i]; },
                [&](int i, float acc, float ai) { pc[i] = -acc * ai; }, a.sellColBase);
        };
        if (a.sellMaxW <= 5) h1(std::integral_constant<int, 5>{});
        else h1(std::integral_constant<int, 6>{});
        if (!t.barrier(where++)) return false;
        }
        // H2: p_1 and q_1 = S p_1, p.q
        float pqHi = 0.f, pqLo = 0.f;
        auto e2 = [&](int row, float acc, float pi) {
            pc[row] = pi;
            if constexpr (Resident) sq1[row - b0] = acc;
            else a.q32[row] = acc;
            df_acc(pqHi, pqLo, pi, acc);
        };
        if constexpr (Schur) {
            // every column of S is a colour-1 unknown: p_j = z_j + beta p_j on the fly
            auto gs = [&](int c) { return fmaf(betaf, pp[c], w[c]); };
            auto pre = [&](int row) { return DiffPre<float>{gs(row), F.sRowsum32[row]}; };
            auto fin = [&](int row, float acc, const DiffPre<float>& q) { e2(row, fmaf(q.rs, q.self, acc), q.self); };
            sell_rows<float, float, true, 1, 9, unsigned short>(F.sStart, F.sCol16, F.sVal32, b0, b1, gs, pre, fin,
                                                                 F.sColBase);
        } else {
            auto g2 = [&](int c) { return c >= c1 ? fmaf(betaf, pp[c], w[c]) : pc[c]; };
            if (a.sellMaxW <= 5) product32<false, 5, C16>(nullptr, a, b0, b1, nullptr, g2, e2);
            else product32<false, 6, C16>(nullptr, a, b0, b1, nullptr, g2, e2);
        }
        const double pq = block_sum_df(pqHi, pqLo, smem);
        if (threadIdx.x == 0) a.partials[t.rank] = pq;
        if (!t.barrier(where++)) return false;
        {
            const double pqs = grid_sum0(a.partials, G);
            if (threadIdx.x == 0) {
                const bool bad = !(pqs > 0.0) || isinf(pqs);
                decision_put(smem, bad ? 0.f : (float)(L.rz / pqs), bad);
            }
        }
        const Decision da = decision_get(smem);
        if (da.code) { L.innerBreakdown = 1; break; }
        const float alphaf = da.v;
        const bool fold = fold_iteration(L);
        // U, colour-0 rows: d_0 += alpha u_0, so that x_0 follows the directions q_1 was formed with (the rounded
        // u_0), not their exact projection; the refresh then finds the residual the recurrence carries
        if constexpr (!Schur) {
            for (int i = a0 + (int)threadIdx.x; i < a1; i += bs) {
                if constexpr (Resident) sd0[i - a0] = fold_correction(a, i, fmaf(alphaf, pc[i], sd0[i - a0]), fold, invScale);
                else a.d32[i] = fold_correction(a, i, fmaf(alphaf, pc[i], a.d32[i]), fold, invScale);
            }
        }
        // U: colour-1 rows
        float rrHi = 0.f, rrLo = 0.f;
        DotAcc<float> rzn;
        for (int i0 = b0 + (int)threadIdx.x; i0 < b1; i0 += kRowsLean * bs) {
            float pi[kRowsLean], qi[kRowsLean], di[kRowsLean], ri[kRowsLean], vi[kRowsLean];
#pragma unroll
            for (int u = 0; u < kRowsLean; ++u) {
                const int i = i0 + u * bs;
                if (i < b1) {
                    pi[u] = pc[i];
                    if constexpr (Resident) {
                        qi[u] = sq1[i - b0];
                        di[u] = sd1[i - b0];
                        ri[u] = sr1[i - b0];
                    } else {
                        qi[u] = a.q32[i];
                        di[u] = a.d32[i];
                        ri[u] = r[i];
                    }
                    if constexpr (Resident && Schur) vi[u] = sv1[i - b0];
                    else vi[u] = dinv[i];
                }
            }
#pragma unroll
            for (int u = 0; u < kRowsLean; ++u) {
                const int i = i0 + u * bs;
                if (i < b1) {
                    const float dn = fold_correction(a, i, fmaf(alphaf, pi[u], di[u]), fold, invScale);
                    const float rn = fmaf(-alphaf, qi[u], ri[u]);
                    if constexpr (Resident) {
                        sd1[i - b0] = dn;
                        sr1[i - b0] = rn;
                    } else {
                        a.d32[i] = dn;
                        r[i] = rn;
                    }
                    df_acc(rrHi, rrLo, rn, rn);
                    const float z = (rn * vi[u]) * vi[u];
                    w[i] = z;
                    rzn.add(rn, z);
                }
            }
        }
        const double rrn = block_sum_df(rrHi, rrLo, smem);
        const double rzb = rzn.block(smem);
        if (threadIdx.x == 0) {
            a.partials[G + t.rank] = rrn;
            a.partials[4 * G + t.rank] = rzb;
        }
        if (!t.barrier(where++)) return false;
        const double rrs = grid_sum(a.partials + G, G, smem);
        const double rzs = grid_sum(a.partials + 4 * G, G, smem);
        ++L.it;
        L.flip ^= 1;
        if (!(rrs == rrs) || isinf(rrs)) { L.innerBreakdown = 1; break; }
        if (rrs <= rrStop) break;   // time for a true residual
        if (L.it - L.itRef >= kMaxInnerBetweenRefresh) break;
        if (!(rzs > 0.0) || isinf(rzs)) { L.innerBreakdown = 1; break; }
        L.beta = block_scalar(smem, [&] { return rzs / L.rz; });
        L.rz = rzs;
        betaf = (float)L.beta;
    }
    if constexpr (Resident) {   // d of every own row back to its global copy (the refresh folds it into x)
        __syncthreads();
        for (int k = threadIdx.x; k < n1; k += bs) a.d32[b0 + k] = sd1[k];
        if constexpr (!Schur)
            for (int k = threadIdx.x; k < n0; k += bs) a.d32[a0 + k] = sd0[k];
    }
    L.state = kLoopRefresh;
    return true;
}

// The end of a mixed PCG solve (state kLoopDone): when it stopped short of the tolerance with budget left, plain
// FP64 CG from the current iterate with the plain method's own budget; then the solve's info.
template <bool Wide = false>
static __device__ int pcg_mixed_finish(Team& t, const CgArgs& a, double* stage, double* smem, const PcgLoop& L) {
    if (L.status == NSF_ERR_NOT_CONVERGED && (a.fallbackMaxIt > 0 || L.it < a.maxIt)) {
        CgArgs f = a;
        f.bRowptr = nullptr;
        f.b = a.b;
        f.x0 = a.x;
        f.maxIt = a.fallbackMaxIt > 0 ? a.fallbackMaxIt : a.maxIt - L.it;
        const int fst = team_cg_fp64<Wide>(t, f, stage, smem);
        if (fst == NSF_ERR_BARRIER_TIMEOUT) return fst;
        if (t.rank == 0 && threadIdx.x == 0) {
            a.info->iterations += L.it;
            a.info->outer = L.refresh;
            a.info->fallback = 1;
        }
        return fst;
    }
    write_info(t, a, L.it, L.status, L.refresh, L.rr64, L.bb);
    return L.status;
}

// The whole mixed PCG solve in one persistent launch.
template <bool Wide = false>
static __device__ int pcg_mixed_body(Team& t, const CgArgs& a, double* stage, double* smem, SellRing* ring) {
    PcgLoop L;
    pcg_loop_init(L);
    int where = 300;
    while (true) {
        if (!pcg_mixed_refresh<Wide>(t, a, stage, smem, ring, L, where) ||
            (L.state == kLoopInner && !pcg_mixed_inner<Wide>(t, a, stage, smem, ring, L, where))) {
            write_info(t, a, L.it, NSF_ERR_BARRIER_TIMEOUT, L.refresh, L.rr64, L.bb);
            return NSF_ERR_BARRIER_TIMEOUT;
        }
        if (L.state == kLoopDone) break;
    }
    return pcg_mixed_finish<Wide>(t, a, stage, smem, L);
}

// Preconditioned solves of the caller's system: permute in, solve the colour-permuted system, permute out.
// (The solve works on the kernel's own argument block: the permuted vectors are passed in it, so no copy of the
// arguments lands in local memory.)
template <bool Wide = false>
static __device__ int team_pcg_fp64(Team& t, const CgArgs& a, double* stage, double* smem) {
    int where = 190;
    if (!permute_in<Wide>(t, a, stage, where)) {
        write_info(t, a, 0, NSF_ERR_BARRIER_TIMEOUT, 0, 0, 0);
        return NSF_ERR_BARRIER_TIMEOUT;
    }
    const int st = pcg_fp64_body<Wide>(t, a, stage, smem);
    if (st != NSF_ERR_BARRIER_TIMEOUT) permute_out(t, a);
    return st;
}

template <bool Wide = false>
static __device__ int team_pcg_mixed(Team& t, const CgArgs& a, double* stage, double* smem, SellRing* ring = nullptr) {
    int where = 190;
    if (!permute_in<Wide>(t, a, stage, where)) {
        write_info(t, a, 0, NSF_ERR_BARRIER_TIMEOUT, 0, 0, 0);
        return NSF_ERR_BARRIER_TIMEOUT;
    }
    const int st = pcg_mixed_body<Wide>(t, a, stage, smem, ring);
    if (st != NSF_ERR_BARRIER_TIMEOUT) permute_out(t, a);
    return st;
}

// The split form (narrow matrices; a.loop holds the state between launches).  Refresh launch: on the first, the
// permutation in and a fresh state; a true-residual refresh; when the solve is done, its end and the permutation
// out.  Inner launch: FP32 iterations up to the next refresh.  State and info are written by thread 0 of block 0
// (every thread holds the same state).
static __device__ void pcg_loop_store(const Team& t, const CgArgs& a, const PcgLoop& L) {
    if (t.rank == 0 && threadIdx.x == 0) *a.loop = L;
}

static __device__ void team_pcg_mixed_refresh(Team& t, const CgArgs& a, double* stage, double* smem, SellRing* ring) {
    int where = 190;
    PcgLoop L;
    if (a.loopInit) {
        pcg_loop_init(L);
        if (!permute_in<false>(t, a, stage, where)) {
            write_info(t, a, 0, NSF_ERR_BARRIER_TIMEOUT, 0, 0, 0);
            L.state = kLoopDone;
            pcg_loop_store(t, a, L);
            return;
        }
    } else {
        L = *a.loop;
    }
    if (!(a.f.reduced ? pcg_mixed_refresh_reduced<false>(t, a, stage, smem, L, where)
                      : pcg_mixed_refresh<false>(t, a, stage, smem, ring, L, where))) {
        write_info(t, a, L.it, NSF_ERR_BARRIER_TIMEOUT, L.refresh, L.rr64, L.bb);
        L.state = kLoopDone;
        pcg_loop_store(t, a, L);
        return;
    }
    if (L.state == kLoopDone) {
        const int st = pcg_mixed_finish<false>(t, a, stage, smem, L);
        if (st != NSF_ERR_BARRIER_TIMEOUT) permute_out(t, a);
    }
    pcg_loop_store(t, a, L);
}

// The reduced form's inner launch (two colours, a SELL copy and a.f.reduced; see pcg_mixed_inner_reduced).
template <bool C16 = false, bool Resident = false, bool Schur = false>
static __device__ void team_pcg_mixed_inner_reduced(Team& t, const CgArgs& a, double* smem) {
    int where = 400;
    const PcgLoop& G = *a.loop;
    PcgLoop L;
    L.rz = G.rz;
    L.beta = G.beta;
    L.rrRef = G.rrRef;
    L.target = G.target;
    L.scale = G.scale;
    L.it = G.it;
    L.itRef = G.itRef;
    L.flip = G.flip;
    L.rflip = G.rflip;
    const bool ok = pcg_mixed_inner_reduced<C16, Resident, Schur>(t, a, smem, L, where);
    if (!ok) write_info(t, a, L.it, NSF_ERR_BARRIER_TIMEOUT, G.refresh, G.rr64, G.bb);
    if (t.rank == 0 && threadIdx.x == 0) {
        a.loop->rz = L.rz;
        a.loop->beta = L.beta;
        a.loop->it = L.it;
        a.loop->flip = L.flip;
        a.loop->rflip = L.rflip;
        a.loop->innerBreakdown = L.innerBreakdown;
        a.loop->state = ok ? L.state : kLoopDone;
    }
}

// (FusedOnly: the caller guarantees two or more colours; the one-colour loop and its CSR staging are left out.
// Resident: the caller guarantees exactly two colours and dynamic shared memory for the row state.)
template <bool C16 = false, bool FusedOnly = false, bool Resident = false, bool H16 = false>
static __device__ void team_pcg_mixed_inner(Team& t, const CgArgs& a, double* stage, double* smem, SellRing* ring) {
    int where = 400;
    // the fields the inner iterations read or write (the rest of the state stays in memory)
    const PcgLoop& G = *a.loop;
    PcgLoop L;
    L.rz = G.rz;
    L.beta = G.beta;
    L.rrRef = G.rrRef;
    L.target = G.target;
    L.scale = G.scale;
    L.it = G.it;
    L.itRef = G.itRef;
    L.flip = G.flip;
    L.rflip = G.rflip;
    bool ok;
    if constexpr (Resident) ok = pcg_mixed_inner_fused<C16, true, H16>(t, a, stage, smem, ring, L, where);
    else if constexpr (FusedOnly) ok = pcg_mixed_inner_fused<C16, false, H16>(t, a, stage, smem, ring, L, where);
    else ok = a.f.colours >= 2 ? pcg_mixed_inner_fused<C16>(t, a, stage, smem, ring, L, where)
                               : pcg_mixed_inner<false, true>(t, a, stage, smem, ring, L, where);
    if (!ok) write_info(t, a, L.it, NSF_ERR_BARRIER_TIMEOUT, G.refresh, G.rr64, G.bb);
    if (t.rank == 0 && threadIdx.x == 0) {
        a.loop->rz = L.rz;
        a.loop->beta = L.beta;
        a.loop->it = L.it;
        a.loop->flip = L.flip;
        a.loop->rflip = L.rflip;
        a.loop->innerBreakdown = L.innerBreakdown;
        a.loop->state = ok ? L.state : kLoopDone;
    }
}

}  // namespace nsf
