// batched_ls.cuh — least squares over a batch of small, uneven problems,
// one warp per problem.
//
// After the batched factorization (batched.cuh) every problem p holds its R
// and reflectors (as RNP::LA::QR::Factor leaves them, RNP/LA/QR.hpp:129-197)
// at its offset of the packed buffer.  One warp then solves the problem:
//   plain : x = R^{-1} (Q^H b)(0:n)   (MultQ "L","C", RNP/LA/QR.hpp:337-429,
//           then the upper triangular solve of BLAS::SolveTrM,
//           RNP/BLAS/BLAS_mix.hpp:2096-2113), in the working precision;
//   mixed : the same steps on a low-precision (FP32) factorization as the
//           correction equation of an iterative refinement whose residual
//           r = b - A x, solution x and error metrics are FP64:
//             Q step:    x += R^{-1} (Q^H r)(0:n)
//             CSNE step: x += R^{-1} R^{-H} A^H r   (corrected seminormal
//                        equations, when the Q steps stall above the bound)
//           stopping when the LS backward error estimate
//           mu = ||R^{-H} A^H r|| / ||x|| and the normal residual
//           eta = ||A^H r|| / (||A||_F (||A||_F ||x|| + ||b||)) are both
//           below 10 n eps, or the correction stops shrinking.
// Lane l holds rows l, l+32, ... of the m-vectors in registers (MT slots,
// m <= 32 MT); the FP32 column sweeps (reflector application, triangular
// solves) load the next column while the current one is used, the FP64
// sweeps (residual, A^H r) are bound by FP64 throughput instead.
#pragma once
#include "batched.cuh"
#include "ls_kernels.cuh"

namespace rnpgpu {

template <class TH, class TL> struct LsBatchArgs {
    const BatchDesc *desc;
    int count;
    const TH *A;    // FP64 problem matrices (mixed) or null (plain)
    const TL *F;    // factorizations (R and reflectors), same offsets as A
    const TL *tau;  // their tau
    const TH *B;    // right-hand sides at b_off
    TH *X;          // solutions at x_off
    int refine;     // 0: plain solve in TL (= TH); 1: mixed refinement
    int max_iter;
    int *iters;     // per problem (by index), may be null
    double *berr;   // per problem: mu (mixed) , may be null
    double *eta;    // per problem: eta (mixed), may be null
    unsigned *queue;
};

template <class T> __device__ __forceinline__ T vcol(const T *F, int lda, int i, int j, int m) {
    // column j of V in stored form: 0 above the diagonal, 1 on it, 0 past m
    if (i > j && i < m) return F[i + (size_t)j * lda];
    return (i == j) ? T(1) : T(0);
}

template <class TH, class TL, int MT> __device__ void ls_problem(const LsBatchArgs<TH, TL> &q, const BatchDesc &d) {
    const int lane = threadIdx.x & 31;
    const int m = d.m, n = d.n, lda = d.lda;
    const TL *F = q.F + d.a_off;
    const TL *tp = q.tau + d.tau_off;
    const TH *bp = q.B + d.b_off;
    TH *xp = q.X + d.x_off;
    const TH *Ap = q.refine ? q.A + d.a_off : nullptr;

    // the next column is loaded during the current one where registers allow
    constexpr bool kPre = sizeof(TL) * MT <= 128;
    TL y[MT];
    // y <- Q^H y, reflectors 0..n-1 in order (H_j^H = I - conj(tau_j) v v^H)
    auto apply_qh = [&]() {
        TL vn[MT], taun = TL(0);
        if (kPre) {
#pragma unroll
            for (int t = 0; t < MT; ++t) vn[t] = vcol(F, lda, lane + 32 * t, 0, m);
            taun = tp[0];
        }
        for (int j = 0; j < n; ++j) {
            TL v[MT], tj;
            if (kPre) {
#pragma unroll
                for (int t = 0; t < MT; ++t) v[t] = vn[t];
                tj = taun;
                if (j + 1 < n) {
#pragma unroll
                    for (int t = 0; t < MT; ++t) vn[t] = vcol(F, lda, lane + 32 * t, j + 1, m);
                    taun = tp[j + 1];
                }
            } else {
#pragma unroll
                for (int t = 0; t < MT; ++t) v[t] = vcol(F, lda, lane + 32 * t, j, m);
                tj = tp[j];
            }
            TL s = TL(0);
#pragma unroll
            for (int t = 0; t < MT; ++t) s = fmac(Tr<TL>::conj(v[t]), y[t], s);
            s = warp_sum(s) * Tr<TL>::conj(tj);
#pragma unroll
            for (int t = 0; t < MT; ++t) y[t] = fmac(-v[t], s, y[t]);
        }
    };
    // y(0:n) <- R^{-1} y(0:n) (backward substitution, column-oriented; the
    // next column of R is loaded while the current one is used)
    auto load_rcol = [&](int j, TL (&col)[MT], TL &dg) {
#pragma unroll
        for (int u = 0; u < MT; ++u) {
            const int i = lane + 32 * u;
            col[u] = (j >= 0 && i < j) ? F[i + (size_t)j * lda] : TL(0);
        }
        dg = (j >= 0) ? F[j + (size_t)j * lda] : TL(1);
    };
    auto solve_r = [&]() {
        TL cn[MT], dn = TL(1);
        if (kPre) load_rcol(n - 1, cn, dn);
#pragma unroll
        for (int t = MT - 1; t >= 0; --t) {
            if (32 * t >= n) continue;
            for (int jl = 31; jl >= 0; --jl) {
                const int j = 32 * t + jl;
                if (j >= n) continue;
                TL col[MT], dg;
                if (kPre) {
#pragma unroll
                    for (int u = 0; u < MT; ++u) col[u] = cn[u];
                    dg = dn;
                    load_rcol(j - 1, cn, dn);
                } else {
                    load_rcol(j, col, dg);
                }
                const TL dj = shfl(y[t], jl) / dg;
                if (lane == jl) y[t] = dj;
#pragma unroll
                for (int u = 0; u < MT; ++u)
                    if (u <= t) y[u] = fmac(-col[u], dj, y[u]);
            }
        }
    };
    // y(0:n) <- R^{-H} y(0:n) (forward substitution with the conjugate
    // transpose; row j of R right of the diagonal, the next row prefetched)
    auto load_rrow = [&](int j, TL (&row)[MT], TL &dg) {
#pragma unroll
        for (int u = 0; u < MT; ++u) {
            const int i = lane + 32 * u;
            row[u] = (j < n && i > j && i < n) ? Tr<TL>::conj(F[j + (size_t)i * lda]) : TL(0);
        }
        dg = (j < n) ? Tr<TL>::conj(F[j + (size_t)j * lda]) : TL(1);
    };
    auto solve_rh = [&]() {
        TL rn[MT], dn = TL(1);
        if (kPre) load_rrow(0, rn, dn);
#pragma unroll
        for (int t = 0; t < MT; ++t) {
            if (32 * t >= n) continue;
            for (int jl = 0; jl < 32; ++jl) {
                const int j = 32 * t + jl;
                if (j >= n) break;
                TL row[MT], dg;
                if (kPre) {
#pragma unroll
                    for (int u = 0; u < MT; ++u) row[u] = rn[u];
                    dg = dn;
                    load_rrow(j + 1, rn, dn);
                } else {
                    load_rrow(j, row, dg);
                }
                const TL dj = shfl(y[t], jl) / dg;
                if (lane == jl) y[t] = dj;
#pragma unroll
                for (int u = 0; u < MT; ++u)
                    if (u >= t) y[u] = fmac(-row[u], dj, y[u]);
            }
        }
    };

    // a batch in one precision only ever takes the plain solve, and the
    // refinement is compiled for mixed precisions only (the plain kernels
    // keep their registers for the solve)
    if (std::is_same<TH, TL>::value || !q.refine) {
        // plain: x = R^{-1} (Q^H b)(0:n) in the working precision
#pragma unroll
        for (int t = 0; t < MT; ++t) {
            const int i = lane + 32 * t;
            y[t] = (i < m) ? convert_scalar<TH, TL>(bp[i]) : TL(0);
        }
        apply_qh();
        solve_r();
#pragma unroll
        for (int t = 0; t < MT; ++t) {
            const int i = lane + 32 * t;
            if (i < n) xp[i] = convert_scalar<TL, TH>(y[t]);
        }
        if (q.iters && lane == 0) q.iters[d.index] = 0;
        return;
    }

    if constexpr (!std::is_same<TH, TL>::value) {
    // ---- mixed refinement
    TH r[MT];
    double bn2 = 0.0;
#pragma unroll
    for (int t = 0; t < MT; ++t) {
        const int i = lane + 32 * t;
        r[t] = (i < m) ? bp[i] : TH(0);
        bn2 += abs2(r[t]);
        if (i < n) xp[i] = TH(0);
    }
    bn2 = warp_sum(bn2);
    __syncwarp();
    double an2 = -1.0;  // ||A||_F^2, from the first residual sweep
    // r = b - A x (FP64), column by column (FP64 throughput bounds this
    // sweep, not the load latency)
    auto residual = [&]() {
        double a2 = 0.0;
        // the ||A||_F test once, not per element (FP64 compares share the
        // slow FP64 pipe)
        const bool first = an2 < 0.0;
#pragma unroll
        for (int t = 0; t < MT; ++t) {
            const int i = lane + 32 * t;
            r[t] = (i < m) ? bp[i] : TH(0);
        }
        for (int j = 0; j < n; ++j) {
            const TH xj = xp[j];
            const TH *aj = Ap + (size_t)j * lda;
#pragma unroll
            for (int t = 0; t < MT; ++t) {
                const int i = lane + 32 * t;
                const TH a = (i < m) ? aj[i] : TH(0);
                r[t] = fmac(-a, xj, r[t]);
                if (first) a2 += abs2(a);
            }
        }
        if (first) an2 = warp_sum(a2);
    };
    // g = A^H r (FP64) into y as TL (g kept in FP64 only for its norm)
    double gn2 = 0.0;
    auto normal_eq = [&]() {
        double g2 = 0.0;
#pragma unroll
        for (int t = 0; t < MT; ++t) y[t] = TL(0);
        // 16 columns at a time: every lane's partial dot products over its
        // rows, then one butterfly over the warp (16 adds for 16 columns
        // instead of a 32-lane reduction per column); lanes 2e and 2e+1 end
        // with column 16 g + e, which lane (16 g + e) % 32 keeps in y
        for (int g = 0; 16 * g < n; ++g) {
            TH acc[16];
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int j = 16 * g + e;
                TH s = TH(0);
                if (j < n) {
                    const TH *aj = Ap + (size_t)j * lda;
#pragma unroll
                    for (int t = 0; t < MT; ++t) {
                        const int i = lane + 32 * t;
                        const TH a = (i < m) ? aj[i] : TH(0);
                        s = fmac(Tr<TH>::conj(a), r[t], s);
                    }
                }
                acc[e] = s;
            }
            const int e = warp_reduce16(acc, lane);
            if ((lane & 1) == 0 && 16 * g + e < n) g2 += abs2(acc[0]);
            const TL got = shfl(convert_scalar<TH, TL>(acc[0]), 2 * (lane & 15));
            const bool mine = (lane >> 4) == (g & 1) && 16 * g + (lane & 15) < n;
#pragma unroll
            for (int t = 0; t < MT; ++t)
                if (mine && t == (g >> 1)) y[t] = got;
        }
        gn2 = warp_sum(g2);
    };
    const double eps = 0x1p-52;
    const double tol = 10.0 * (double)n * eps;
    double xn2 = 0.0, dn2 = 0.0, mu = HUGE_VAL, eta = HUGE_VAL;
    // x += d with d in y(0:n); returns ||d||^2, sets ||x||^2
    auto add_correction = [&]() {
        double d2 = 0.0, x2 = 0.0;
#pragma unroll
        for (int t = 0; t < MT; ++t) {
            const int i = lane + 32 * t;
            if (i < n) {
                const TH nx = xp[i] + convert_scalar<TL, TH>(y[t]);
                xp[i] = nx;
                d2 += abs2(y[t]);
                x2 += abs2(nx);
            }
        }
        __syncwarp();
        xn2 = warp_sum(x2);
        return warp_sum(d2);
    };
    auto check = [&]() {
        normal_eq();  // y = A^H r
        solve_rh();   // y = R^{-H} A^H r
        double t2 = 0.0;
#pragma unroll
        for (int t = 0; t < MT; ++t) {
            const int i = lane + 32 * t;
            if (i < n) t2 += abs2(y[t]);
        }
        t2 = warp_sum(t2);
        const double xn = sqrt(xn2), an = sqrt(an2);
        mu = xn > 0.0 ? sqrt(t2) / xn : 0.0;
        const double den = an * (an * xn + sqrt(bn2));
        eta = den > 0.0 ? sqrt(gn2) / den : 0.0;
        // a non-finite x or product never passes the test
        if (!isfinite(xn + t2 + den + gn2)) mu = eta = nan("");
    };

    bool csne = false, checked = false;
    double prev = HUGE_VAL;
    int it = 0;
    for (it = 0; it < q.max_iter;) {
        if (!csne) {
#pragma unroll
            for (int t = 0; t < MT; ++t) y[t] = convert_scalar<TH, TL>(r[t]);
            apply_qh();
        }
        // (CSNE: y already holds R^{-H} A^H r from the last check)
        solve_r();
        dn2 = add_correction();
        residual();
        ++it;
        const double corr = xn2 > 0.0 ? sqrt(dn2 / xn2) : (dn2 > 0.0 ? HUGE_VAL : 0.0);
        const bool stagnated = it >= 2 && corr > (csne ? 0.9 : 0.5) * prev;
        const bool last = it == q.max_iter;
        prev = corr;
        checked = false;
        if (corr <= 1e-5 || stagnated || last || csne) {
            check();
            checked = true;
            const bool ok = mu <= tol && eta <= tol;
            if (ok || last) break;
            if (!csne) {
                csne = true;
                prev = HUGE_VAL;
            } else if (stagnated || corr <= 2.0 * eps) {
                break;
            }
        }
    }
    if (!checked) check();
    if (lane == 0) {
        if (q.iters) q.iters[d.index] = it;
        if (q.berr) q.berr[d.index] = mu;
        if (q.eta) q.eta[d.index] = eta;
    }
    }
}

// persistent warps: each takes the next problem from the work queue (the
// descriptors are sorted by decreasing cost)
template <class TH, class TL, int MT> __global__ void __launch_bounds__(256, 1) k_ls_batched(LsBatchArgs<TH, TL> q) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned idx = 0;
        if (lane == 0) idx = atomicAdd(q.queue, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= (unsigned)q.count) break;
        const BatchDesc d = q.desc[idx];
        ls_problem<TH, TL, MT>(q, d);
    }
}

// flat element-wise conversion of a packed buffer
template <class Tin, class Tout> __global__ void __launch_bounds__(256) k_convert_flat(size_t count, const Tin *src, Tout *dst) {
    for (size_t e = (size_t)blockIdx.x * 256 + threadIdx.x; e < count; e += (size_t)gridDim.x * 256) dst[e] = convert_scalar<Tin, Tout>(src[e]);
}

} // namespace rnpgpu
