// =============================================================================
// batch_implicit.cu -- linear solves of the batched Rosenbrock integrator:
// (I - g J(N)) x = r for every cell at once, g = gamma dt, by GMRES(m)
// (a cell's solve may end early at a relative residual tol, and cells above
// tol after m steps may restart on r - A x), right-preconditioned by the
// diagonal
// P_i = 1 + g (sum_k beta_ik N_k + beta_ii N_i + S_i [N_i guarded]), i.e. the
// loss part of -J_ii (death and breakage; the birth terms are left out).
// J is never formed: each Arnoldi step takes one Jacobian-vector product
// (two passes of the pair kernel, batch_jvp_prep + batch_main).
//
// One CTA per cell for the vector work (n <= a few thousand bins per cell:
// the cell's vectors stay in L1/L2); all inner products are fixed-order block
// sums, so a solve is bitwise reproducible. The small per-cell Hessenberg
// least-squares problem is updated with Givens rotations by thread 0.
// =============================================================================
#include "batch_internal.cuh"
#include "agg_tile.cuh"

namespace pbe_gb300 {
namespace {

// beta(x_i, x_i) of the aggregation kernels (src/aggregation_kernels.cuh:56-89
// at x_j = x_k): a_i / a_i + a_i / a_i + 2 = 4 and (2 a_i)^3 = 8 x_i.
template <int K>
__device__ __forceinline__ double beta_self(double xi, double b0, double bbr, double bsh)
{
    if constexpr (K == 0) return b0;
    else if constexpr (K == 1) return b0 * (2.0 * xi);
    else if constexpr (K == 2) return b0 * (xi * xi);
    else if constexpr (K == 3) return 4.0 * bbr;
    else if constexpr (K == 4) return 8.0 * bsh * xi;
    else return fma(8.0 * bsh, xi, 4.0 * bbr);
}

__device__ __forceinline__ double sel_value_i(int F, double v, double S0, double v_ref,
                                              double alpha, double v_min)
{
    switch (F) {
    case 0: return selection<0>(v, S0, v_ref, alpha, v_min);
    case 1: return selection<1>(v, S0, v_ref, alpha, v_min);
    case 2: return selection<2>(v, S0, v_ref, alpha, v_min);
    default: return selection<3>(v, S0, v_ref, alpha, v_min);
    }
}

// Start of a cycle: preconditioner, |r|, v_0 = r / |r|, z = P^-1 v_0. The
// first cycle of a solve records |r| and clears the cell's conv flag; a later
// cycle (r = the restart residual) runs only cells without conv.
template <int K>
__global__ void __launch_bounds__(256)
gmres_start_kernel(BatchDev d, GmresDev g, const double* __restrict__ N,
                   const double* __restrict__ r, const pbe_batch_cell_params_t* __restrict__ params,
                   int first)
{
    __shared__ double sh[8];
    __shared__ double m_s[5];
    const int c = blockIdx.x;
    const BatchCellDev cd = d.cells[c];
    const BatchGridDev gd = d.grids[cd.grid];
    const pbe_batch_cell_params_t P = params[c];
    const int off = cd.off, n = cd.n;
    const double* x = d.gx + gd.off;
    const double* a = d.ga + gd.off;
    const double* ia = d.gia + gd.off;
    const bool agg = d.kernel >= 0;
    const double gt = g.gtc ? g.gtc[c] : g.gt;
    if (agg) {
        double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double y = N[off + i];
            m[0] = fma(ia[i], y, m[0]);
            m[1] += y;
            m[2] = fma(a[i], y, m[2]);
            m[3] = fma(a[i] * a[i], y, m[3]);
            m[4] = fma(x[i], y, m[4]);
        }
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            const double s_ = block_sum(m[q], sh);
            if (threadIdx.x == 0) m_s[q] = s_;
        }
        __syncthreads();
    }
    double rr = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double y = N[off + i], xi = x[i];
        double loss = 0.0;
        if (agg) {
            loss = death_factor<K>(xi, a[i], ia[i], m_s, P.beta0, P.beta_br, P.beta_sh)
                 + beta_self<K>(xi, P.beta0, P.beta_br, P.beta_sh) * y;
        }
        if (d.selection >= 0 && d.nq > 0) {
            const double S = d.Sx ? d.Sx[off + i]
                                  : sel_value_i(d.selection, xi, P.S0, P.v_ref, P.alpha, P.v_min);
            if (S != 0.0 && y > kBreakageNMin) loss += S;
        }
        const double p = 1.0 + gt * fmax(loss, 0.0);
        g.P[off + i] = (p == p && p < 1.7e308) ? p : 1.0;
        const double ri = r[off + i];
        rr = fma(ri, ri, rr);
    }
    rr = block_sum(rr, sh);
    const double b0 = sqrt(rr);
    const bool skipped = (g.skip && g.skip[c]) || (!first && g.conv[c]);
    const bool live = b0 > 0.0 && b0 < 1.7e308 && !skipped;
    const double inv = live ? 1.0 / b0 : 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double v0 = live ? r[off + i] * inv : 0.0;
        g.V[off + i] = v0;
        g.Z[off + i] = v0 / g.P[off + i];
    }
    if (threadIdx.x == 0) {
        const int m1 = g.m + 1;
        for (int q = 0; q < m1; ++q) g.gv[c * m1 + q] = 0.0;
        g.gv[c * m1] = live ? b0 : 0.0;
        g.beta0[c] = live ? b0 : 0.0;
        g.kval[c] = 0;
        g.done[c] = live ? 0 : 1;
        if (first) {
            g.rnorm[c] = live ? b0 : 0.0;
            g.conv[c] = live ? 0 : 1;
            g.last[c] = 0.0;
        }
    }
}

// Arnoldi step j of every running cell: w = z - g J z (W holds J z on entry),
// modified Gram-Schmidt against v_0..v_j, v_{j+1} = w / |w|, the new column
// of H rotated into the triangular factor, the residual norm |g_{j+1}|.
__global__ void __launch_bounds__(256)
gmres_arnoldi_kernel(BatchDev d, GmresDev g, int j)
{
    __shared__ double sh[8];
    __shared__ double h_s[kGmresMaxDim + 1];
    __shared__ int more_s;
    const int c = blockIdx.x;
    const BatchCellDev cd = d.cells[c];
    const int off = cd.off, n = cd.n;
    const size_t T = static_cast<size_t>(g.total);
    if (g.done[c]) {                     // converged or exhausted: keep z = 0
        for (int i = threadIdx.x; i < n; i += blockDim.x) g.Z[off + i] = 0.0;
        return;
    }
    double* w = g.W + off;
    const double gt = g.gtc ? g.gtc[c] : g.gt;
    double s0 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double wi = fma(-gt, w[i], g.Z[off + i]);
        w[i] = wi;
        s0 = fma(wi, wi, s0);
    }
    const double wn0 = sqrt(block_sum(s0, sh));      // |A P^-1 v_j| before the projections
    for (int q = 0; q <= j; ++q) {
        const double* vq = g.V + static_cast<size_t>(q) * T + off;
        double s_ = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) s_ = fma(w[i], vq[i], s_);
        const double h = block_sum(s_, sh);
        for (int i = threadIdx.x; i < n; i += blockDim.x) w[i] = fma(-h, vq[i], w[i]);
        if (threadIdx.x == 0) h_s[q] = h;
        __syncthreads();
    }
    double s2 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s2 = fma(w[i], w[i], s2);
    const double hn = sqrt(block_sum(s2, sh));
    if (threadIdx.x == 0) {
        const int m = g.m, m1 = m + 1;
        double* H = g.H + static_cast<size_t>(c) * m1 * m;   // column-major, column j at H + j*m1
        double* col = H + static_cast<size_t>(j) * m1;
        double* cs = g.cs + static_cast<size_t>(c) * m;
        double* sn = g.sn + static_cast<size_t>(c) * m;
        double* gg = g.gv + static_cast<size_t>(c) * m1;
        for (int q = 0; q <= j; ++q) col[q] = h_s[q];
        col[j + 1] = hn;
        for (int q = 0; q < j; ++q) {
            const double t0 = col[q], t1 = col[q + 1];
            col[q] = fma(cs[q], t0, sn[q] * t1);
            col[q + 1] = fma(-sn[q], t0, cs[q] * t1);
        }
        const double rr = hypot(col[j], col[j + 1]);
        const double cj = rr > 0.0 ? col[j] / rr : 1.0;
        const double sj = rr > 0.0 ? col[j + 1] / rr : 0.0;
        cs[j] = cj;
        sn[j] = sj;
        col[j] = rr;
        col[j + 1] = 0.0;
        gg[j + 1] = -sj * gg[j];
        gg[j] = cj * gg[j];
        g.kval[c] = j + 1;
        // a new direction lost to round-off (an invariant Krylov space: the
        // solution is exact), the last allowed step, or a residual |g_{j+1}|
        // within the tolerance ends the cell's solve
        const bool conv = g.tol > 0.0 && fabs(gg[j + 1]) <= g.tol * g.rnorm[c];
        const bool more = hn > 1e-13 * wn0 && j + 1 < g.m && !conv;
        if (!more) g.done[c] = 1;
        more_s = more ? 1 : 0;
    }
    __syncthreads();
    const bool more = more_s != 0;
    const double inv = hn > 0.0 ? 1.0 / hn : 0.0;
    double* v1 = g.V + static_cast<size_t>(j + 1) * T + off;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = more ? w[i] * inv : 0.0;
        v1[i] = v;
        g.Z[off + i] = v / g.P[off + i];
    }
}

// End of a cycle: y = R^-1 g (the kval valid columns), x = P^-1 V y (acc:
// x += P^-1 V y, a restart cycle). A cell that ran this cycle records its
// relative residual |g_k| / |r| (r the system's right-hand side) and, within
// the tolerance, its conv flag; final: resid[c] = max(resid[c], that residual).
__global__ void __launch_bounds__(256)
gmres_finish_kernel(BatchDev d, GmresDev g, double* __restrict__ xo, double* __restrict__ resid,
                    int acc, int final)
{
    __shared__ double y_s[kGmresMaxDim];
    const int c = blockIdx.x;
    const BatchCellDev cd = d.cells[c];
    const int off = cd.off, n = cd.n;
    const int k = g.kval[c];
    const int m = g.m, m1 = m + 1;
    if (threadIdx.x == 0) {
        const double* H = g.H + static_cast<size_t>(c) * m1 * m;
        const double* gg = g.gv + static_cast<size_t>(c) * m1;
        for (int q = k - 1; q >= 0; --q) {
            double s_ = gg[q];
            for (int t = q + 1; t < k; ++t) s_ = fma(-H[static_cast<size_t>(t) * m1 + q], y_s[t], s_);
            const double dq = H[static_cast<size_t>(q) * m1 + q];
            y_s[q] = dq != 0.0 ? s_ / dq : 0.0;
        }
        if (g.beta0[c] > 0.0) {                // the cell ran this cycle
            const double rel = g.rnorm[c] > 0.0 ? fabs(gg[k]) / g.rnorm[c] : 0.0;
            g.last[c] = rel;
            if (g.tol > 0.0 && rel <= g.tol) g.conv[c] = 1;
        }
        if (final && resid) resid[c] = fmax(resid[c], g.last[c]);
    }
    __syncthreads();
    if (acc && k == 0) return;                 // nothing to add
    const size_t T = static_cast<size_t>(g.total);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double s_ = 0.0;
        for (int q = 0; q < k; ++q) s_ = fma(y_s[q], g.V[static_cast<size_t>(q) * T + off + i], s_);
        const double v = s_ / g.P[off + i];
        xo[off + i] = acc ? xo[off + i] + v : v;
    }
}

// Restart residual of every cell without conv: R = r - (x - gamma dt W),
// W = J x on entry.
__global__ void __launch_bounds__(256)
gmres_restart_kernel(BatchDev d, GmresDev g, const double* __restrict__ r,
                     const double* __restrict__ x)
{
    const int c = blockIdx.x;
    if (g.conv[c] || (g.skip && g.skip[c])) return;      // whole block
    const BatchCellDev cd = d.cells[c];
    const double gt = g.gtc ? g.gtc[c] : g.gt;
    for (int i = threadIdx.x; i < cd.n; i += blockDim.x) {
        const int e = cd.off + i;
        g.R[e] = r[e] - fma(-gt, g.W[e], x[e]);
    }
}

// out = a X + b Y over the packed state (Y may be null: out = a X).
__global__ void __launch_bounds__(256)
lincomb_kernel(double* __restrict__ out, double a, const double* __restrict__ X, double b,
               const double* __restrict__ Y, long long total)
{
    for (long long i = blockIdx.x * 256LL + threadIdx.x; i < total; i += 256LL * gridDim.x) {
        const double ax = a * X[i];
        out[i] = Y ? fma(b, Y[i], ax) : ax;
    }
}

// N += c1 K1 + c2 K2 (the Rosenbrock update, summed in that order).
__global__ void __launch_bounds__(256)
ros_update_kernel(double* __restrict__ N, double c1, const double* __restrict__ K1, double c2,
                  const double* __restrict__ K2, long long total)
{
    for (long long i = blockIdx.x * 256LL + threadIdx.x; i < total; i += 256LL * gridDim.x)
        N[i] = N[i] + fma(c1, K1[i], c2 * K2[i]);
}

// Adaptive ROS2. The error estimate is the difference to the embedded
// first-order solution N + dt k1: dt (k1 + k2) / 2. (In this form of the
// method k2 -> -R for small dt, so a first-order combination b1 k1 + b2 k2
// needs b1 - b2 = 1; the only one that also damps infinitely stiff
// components, as ROS2 does, is ROS2's own (3/2, 1/2). The estimate of N + dt k1
// keeps (1/(2 g^2) - 1/g) N of such a component; in practice the stiff
// components sit near their quasi-steady state and the steps stay limited by
// accuracy.)

// Per cell: the second stage's state and gamma dt_c.
__global__ void __launch_bounds__(256)
ros2_stage_kernel(BatchDev d, const double* __restrict__ N, const double* __restrict__ K1,
                  double* __restrict__ Y, double* __restrict__ gtc, Rk45Ctl ctl, double gamma)
{
    const int c = blockIdx.x;
    const BatchCellDev cd = d.cells[c];
    const double dt = ctl.dt[c];           // 0 for a finished cell: Y = N
    for (int i = threadIdx.x; i < cd.n; i += blockDim.x)
        Y[cd.off + i] = fma(dt, K1[cd.off + i], N[cd.off + i]);
    if (threadIdx.x == 0) gtc[c] = gamma * dt;
}

__global__ void __launch_bounds__(256)
ros2_control_kernel(BatchDev d, double* __restrict__ N, const double* __restrict__ K1,
                    const double* __restrict__ K2, Rk45Ctl ctl)
{
    __shared__ double sh[8];
    __shared__ int accept_s;
    const int c = blockIdx.x;
    if (ctl.status[c] != 0) return;                 // whole block
    const BatchCellDev cd = d.cells[c];
    const int off = cd.off, n = cd.n;
    const double dt = ctl.dt[c];
    double s2 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double k1 = K1[off + i], k2 = K2[off + i], y = N[off + i];
        const double yn = y + dt * fma(1.5, k1, 0.5 * k2);
        const double sc = ctl.atol + ctl.rtol * fmax(fabs(y), fabs(yn));
        const double r = (dt * (0.5 * (k1 + k2))) / sc;
        s2 = fma(r, r, s2);
    }
    s2 = block_sum(s2, sh);
    if (threadIdx.x == 0) {
        const double err = sqrt(s2 / n);
        const bool finite = (err == err) && err <= 1.7e308;
        const bool accept = finite && err <= 1.0;
        double fac;
        if (!finite) fac = 0.2;
        else if (err == 0.0) fac = 5.0;
        else fac = fmin(5.0, fmax(0.2, 0.9 / sqrt(err)));
        if (!accept) fac = fmin(fac, 1.0);
        double t = ctl.t[c];
        if (accept) { t += dt; ctl.t[c] = t; ctl.steps[c] += 1; }
        else ctl.rejects[c] += 1;
        const double rem = ctl.t_end - t;
        double nd = fmin(dt * fac, rem);
        int st = 0;
        if (accept && rem <= 1e-12 * fmax(fabs(ctl.t_end), 1.0)) { st = 1; nd = 0.0; }
        else if (nd <= 1e-14 * fmax(fabs(ctl.t_end), 1.0)) { st = 2; nd = 0.0; }
        ctl.dt[c] = nd;
        if (st != 0) { ctl.status[c] = st; atomicAdd(ctl.done, 1); }
        accept_s = accept ? 1 : 0;
    }
    __syncthreads();
    if (accept_s) {
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            N[off + i] = N[off + i] + dt * fma(1.5, K1[off + i], 0.5 * K2[off + i]);
    }
}

template <int K>
cudaError_t start_k(const BatchDev& d, const GmresDev& g, const double* N, const double* r,
                    const pbe_batch_cell_params_t* params, bool first, cudaStream_t s)
{
    gmres_start_kernel<K><<<d.n_cells, 256, 0, s>>>(d, g, N, r, params, first ? 1 : 0);
    return cudaGetLastError();
}

int elementwise_grid(long long total, int num_sms)
{
    const long long b = (total + 255) / 256;
    const long long cap = 8LL * (num_sms > 0 ? num_sms : 1);
    return static_cast<int>(b < 1 ? 1 : (b < cap ? b : cap));
}

} // namespace

cudaError_t batch_gmres_start(const BatchDev& d, const GmresDev& g, const double* N, const double* r,
                              const pbe_batch_cell_params_t* params, bool first, cudaStream_t s)
{
    switch (d.kernel < 0 ? 0 : d.kernel) {
    case 0: return start_k<0>(d, g, N, r, params, first, s);
    case 1: return start_k<1>(d, g, N, r, params, first, s);
    case 2: return start_k<2>(d, g, N, r, params, first, s);
    case 3: return start_k<3>(d, g, N, r, params, first, s);
    case 4: return start_k<4>(d, g, N, r, params, first, s);
    case 5: return start_k<5>(d, g, N, r, params, first, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t batch_gmres_arnoldi(const BatchDev& d, const GmresDev& g, int j, cudaStream_t s)
{
    gmres_arnoldi_kernel<<<d.n_cells, 256, 0, s>>>(d, g, j);
    return cudaGetLastError();
}

cudaError_t batch_gmres_finish(const BatchDev& d, const GmresDev& g, double* x, double* resid,
                               bool acc, bool final, cudaStream_t s)
{
    gmres_finish_kernel<<<d.n_cells, 256, 0, s>>>(d, g, x, resid, acc ? 1 : 0, final ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t batch_gmres_restart(const BatchDev& d, const GmresDev& g, const double* r,
                                const double* x, cudaStream_t s)
{
    gmres_restart_kernel<<<d.n_cells, 256, 0, s>>>(d, g, r, x);
    return cudaGetLastError();
}

cudaError_t batch_lincomb(double* out, double a, const double* X, double b, const double* Y,
                          long long total, int num_sms, cudaStream_t s)
{
    lincomb_kernel<<<elementwise_grid(total, num_sms), 256, 0, s>>>(out, a, X, b, Y, total);
    return cudaGetLastError();
}

cudaError_t batch_ros2_stage(const BatchDev& d, const double* N, const double* K1, double* Y,
                             double* gtc, const Rk45Ctl& ctl, double gamma, cudaStream_t s)
{
    ros2_stage_kernel<<<d.n_cells, 256, 0, s>>>(d, N, K1, Y, gtc, ctl, gamma);
    return cudaGetLastError();
}

cudaError_t batch_ros2_control(const BatchDev& d, double* N, const double* K1, const double* K2,
                               const Rk45Ctl& ctl, cudaStream_t s)
{
    ros2_control_kernel<<<d.n_cells, 256, 0, s>>>(d, N, K1, K2, ctl);
    return cudaGetLastError();
}

cudaError_t batch_ros_update(double* N, double c1, const double* K1, double c2, const double* K2,
                             long long total, int num_sms, cudaStream_t s)
{
    ros_update_kernel<<<elementwise_grid(total, num_sms), 256, 0, s>>>(N, c1, K1, c2, K2, total);
    return cudaGetLastError();
}

} // namespace pbe_gb300
