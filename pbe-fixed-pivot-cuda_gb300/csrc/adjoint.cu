// =============================================================================
// adjoint.cu -- checkpointed discrete adjoint of classical RK4 for one
// instance (pbe_rk4_tape_*; no counterpart in the reference).
//
// Forward: n_steps RK4 steps with the stage arithmetic of the reference
// examples' rk4_step (examples/common/pbe_examples_utils.hpp:416-456); N is
// saved every `every` steps. Backward: for each segment, last first, the
// segment's stage states are recomputed from its checkpoint (every x 4 x n
// doubles), then every step is reversed:
//   a4 = c lam', mu4 = J(Y4)^T a4, a3 = 2c lam' + dt mu4, mu3 = J(Y3)^T a3,
//   a2 = 2c lam' + h mu3, mu2 = J(Y2)^T a2, a1 = c lam' + h mu2,
//   mu1 = J(Y1)^T a1, lam = lam' + mu1 + mu2 + mu3 + mu4,
//   dL/dtheta += sum_q (df/dtheta at Y_q)^T a_q,     h = dt/2, c = dt/6,
// where J^T a is the VJP kernels' dL/dN for lambda = a (vjp.cu). Cost: one
// forward, one recomputed forward and four VJPs per step.
//
// The pivots, quadrature table and coefficient sets do not change during a
// call, so each call first writes the grid-only tables of every parameter set
// (aggregation: cube roots, 1/dx, lag tables, geometric flag; breakage:
// fragment brackets, run starts, the selection function per bin) into that
// set's workspace, and every RHS then recomputes only its N-dependent part
// (agg_stage_launch, brk_stage_launch): bitwise the drop-in calls' result.
// A whole forward and a whole backward call are captured as CUDA graphs (on
// internal copies of N, lambda_T and the gradients, so the caller's pointers
// may change between calls; recaptured when x, t_q or bw_q move);
// PBE_GB300_TAPE_GRAPH=0 launches the kernels one by one instead.
// =============================================================================
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "pbe_internal.cuh"
#include "pbe_gb300.h"

struct pbe_rk4_tape {
    int n = 0, nq = 0, n_steps = 0, every = 1, n_sets = 0, num_sms = 0, device = 0;
    int kernel = -1, selection = -1;
    double dt = 0.0;
    std::vector<pbe_agg_params_t> agg;
    std::vector<pbe_brk_params_t> brk;
    std::vector<int> step_set;
    const double* x = nullptr;
    const double* t_q = nullptr;
    const double* bw_q = nullptr;
    bool recorded = false;
    std::vector<void*> allocs;
    double *ckpt = nullptr, *segY = nullptr, *k = nullptr, *acc = nullptr, *Y = nullptr;
    double *Ncur = nullptr, *lam = nullptr, *lsum = nullptr, *a = nullptr, *mu = nullptr;
    // one aggregation / breakage workspace per parameter set: the grid-only
    // tables (written by a tables pass at the start of every forward and
    // backward call) stay, the stage calls recompute only what depends on N
    std::vector<void*> agg_ws, brk_ws;
    void* vjp_ws = nullptr;
    // whole forward and backward calls captured as CUDA graphs, on internal
    // buffers (Nio, lam_in, gN_out, g_int), keyed by the pivot and quadrature
    // pointers; the caller's arrays are copied in and out around each launch
    bool use_graphs = true;
    cudaStream_t cap = nullptr;
    cudaGraphExec_t fwd_exec = nullptr, bwd_exec = nullptr;
    const double *fwd_key[3] = {nullptr, nullptr, nullptr}, *bwd_key[3] = {nullptr, nullptr, nullptr};
    double *Nio = nullptr, *lam_in = nullptr, *gN_out = nullptr, *g_int = nullptr;
};

namespace pbe_gb300 {
namespace {

// Stage q of one RK4 step (same rounding as the reference's host loop):
// q = 0: acc = k; Y = N + c k.   q = 1, 2: acc += 2 k; Y = N + c k.
// q = 3: acc += k; N += dt6 acc.
__global__ void __launch_bounds__(256)
rk_stage_kernel(double* N, const double* k, double* acc, double* Y, int n, int q, double c,
                double dt6)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double ki = k[i];
    if (q == 0) {
        acc[i] = ki;
        Y[i] = __dadd_rn(N[i], __dmul_rn(c, ki));
    } else if (q < 3) {
        acc[i] = __dadd_rn(acc[i], __dmul_rn(2.0, ki));
        Y[i] = __dadd_rn(N[i], __dmul_rn(c, ki));
    } else {
        const double s = __dadd_rn(acc[i], ki);
        N[i] = __dadd_rn(N[i], __dmul_rn(dt6, s));
    }
}

// a = w lam' (+ c mu), then mu = 0 (ready for the next VJP).
__global__ void __launch_bounds__(256)
adj_coeff_kernel(double* a, const double* lp, double* mu, double w, double c, int n, int first)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[i] = first ? w * lp[i] : fma(c, mu[i], w * lp[i]);
    mu[i] = 0.0;
}

__global__ void __launch_bounds__(256) adj_sum_kernel(double* lsum, const double* mu, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) lsum[i] += mu[i];
}

inline int blocks(int n) { return (n + 255) / 256; }

int set_of(const pbe_rk4_tape* t, int s) { return t->step_set.empty() ? 0 : t->step_set[s]; }

// Grid-only tables of every parameter set (pivots, quadrature table and
// coefficients are fixed for the duration of a forward or backward call).
cudaError_t tables(pbe_rk4_tape* t, const double* N, cudaStream_t s)
{
    cudaError_t e = cudaSuccess;
    for (int m = 0; m < t->n_sets && e == cudaSuccess; ++m) {
        if (t->kernel >= 0) {
            const pbe_agg_params_t& p = t->agg[m];
            AggArgs a{N, t->x, t->k, t->n, t->kernel, p.beta0, p.beta_br, p.beta_sh};
            e = agg_tables_launch(a, t->agg_ws[m], t->num_sms, s);
        }
        if (e == cudaSuccess && t->selection >= 0) {
            const pbe_brk_params_t& p = t->brk[m];
            BrkArgs b{N, t->x, t->t_q, t->bw_q, t->k, t->n, t->nq, t->selection, p.S0, p.v_ref,
                      p.alpha, p.v_min};
            e = brk_tables_launch(b, t->brk_ws[m], s);
        }
    }
    return e;
}

// k = RHS(Yin) with parameter set m, on the set's workspaces (bitwise the
// result of the drop-in calls in gather mode).
cudaError_t rhs(pbe_rk4_tape* t, int m, const double* Yin, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(t->k, 0, sizeof(double) * t->n, s);
    if (e == cudaSuccess && t->kernel >= 0) {
        const pbe_agg_params_t& p = t->agg[m];
        AggArgs a{Yin, t->x, t->k, t->n, t->kernel, p.beta0, p.beta_br, p.beta_sh};
        e = agg_stage_launch(a, false, t->agg_ws[m], t->num_sms, s);
    }
    if (e == cudaSuccess && t->selection >= 0) {
        const pbe_brk_params_t& p = t->brk[m];
        BrkArgs b{Yin, t->x, t->t_q, t->bw_q, t->k, t->n, t->nq, t->selection, p.S0, p.v_ref,
                  p.alpha, p.v_min};
        e = brk_stage_launch(b, t->brk_ws[m], s);
    }
    return e;
}

// One RK4 step on N; Ys (nullable): stage states Y1..Y4 are written to Ys[q n].
cudaError_t step(pbe_rk4_tape* t, int m, double* N, double* Ys, cudaStream_t s)
{
    const double h = 0.5 * t->dt, dt6 = t->dt / 6.0;
    const double cs[4] = {h, h, t->dt, 0.0};
    const size_t un = static_cast<size_t>(t->n);
    cudaError_t e = cudaSuccess;
    if (Ys) e = cudaMemcpyAsync(Ys, N, sizeof(double) * un, cudaMemcpyDeviceToDevice, s);
    for (int q = 0; q < 4 && e == cudaSuccess; ++q) {
        const double* in = (q == 0) ? N : (Ys ? Ys + q * un : t->Y);
        e = rhs(t, m, in, s);
        if (e != cudaSuccess) break;
        double* Yout = (q < 3) ? (Ys ? Ys + (q + 1) * un : t->Y) : t->Y;
        rk_stage_kernel<<<blocks(t->n), 256, 0, s>>>(N, t->k, t->acc, Yout, t->n, q, cs[q], dt6);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t vjp(pbe_rk4_tape* t, int m, const double* Yq, double* g_agg, double* g_brk,
                cudaStream_t s)
{
    cudaError_t e = cudaSuccess;
    if (t->kernel >= 0) {
        const pbe_agg_params_t& p = t->agg[m];
        AggVjpArgs a{Yq, t->x, t->a, t->mu, g_agg + 3 * m, t->n, t->kernel, p.beta0, p.beta_br,
                     p.beta_sh};
        e = agg_vjp_stage_launch(a, t->vjp_ws, t->num_sms, s);
    }
    if (e == cudaSuccess && t->selection >= 0) {
        const pbe_brk_params_t& p = t->brk[m];
        BrkVjpArgs b{Yq, t->x, t->t_q, t->bw_q, t->a, t->mu, g_brk + 4 * m, t->n, t->nq,
                     t->selection, p.S0, p.v_ref, p.alpha, p.v_min};
        // the set's breakage tables (written by tables()): S per bin, fragment brackets
        BrkWs bw;
        brk_ws_layout(t->n, t->nq, static_cast<char*>(t->brk_ws[m]), &bw);
        e = brk_vjp_launch(b, t->vjp_ws, s, bw.Ssel, bw.lo);
    }
    return e;
}

cudaError_t enqueue_forward(pbe_rk4_tape* t, double* N, cudaStream_t s)
{
    const size_t un = static_cast<size_t>(t->n);
    cudaError_t e = tables(t, N, s);
    for (int st = 0; st < t->n_steps && e == cudaSuccess; ++st) {
        if (st % t->every == 0)
            e = cudaMemcpyAsync(t->ckpt + (st / t->every) * un, N, sizeof(double) * un,
                                cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = step(t, set_of(t, st), N, nullptr, s);
    }
    return e;
}

cudaError_t enqueue_backward(pbe_rk4_tape* t, const double* lamT, double* gN0, double* g_agg,
                             double* g_brk, cudaStream_t s)
{
    const size_t un = static_cast<size_t>(t->n);
    const double h = 0.5 * t->dt, c6 = t->dt / 6.0;
    const double cs[3] = {h, h, t->dt};
    double* lam = t->lam;
    double* lsum = t->lsum;
    cudaError_t e = tables(t, t->ckpt, s);
    if (e == cudaSuccess && t->kernel >= 0) {
        // the VJP's grid-only tables (they depend on the pivots alone)
        const pbe_agg_params_t& p = t->agg[0];
        AggVjpArgs a{t->ckpt, t->x, lam, t->mu, g_agg, t->n, t->kernel, p.beta0, p.beta_br,
                     p.beta_sh};
        e = agg_vjp_tables_launch(a, t->vjp_ws, t->num_sms, s);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(lam, lamT, sizeof(double) * un, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && t->kernel >= 0)
        e = cudaMemsetAsync(g_agg, 0, sizeof(double) * 3 * t->n_sets, s);
    if (e == cudaSuccess && t->selection >= 0)
        e = cudaMemsetAsync(g_brk, 0, sizeof(double) * 4 * t->n_sets, s);
    const int nseg = (t->n_steps + t->every - 1) / t->every;
    for (int g = nseg - 1; g >= 0 && e == cudaSuccess; --g) {
        const int s0 = g * t->every, s1 = std::min(s0 + t->every, t->n_steps);
        e = cudaMemcpyAsync(t->Ncur, t->ckpt + g * un, sizeof(double) * un,
                            cudaMemcpyDeviceToDevice, s);
        for (int st = s0; st < s1 && e == cudaSuccess; ++st)
            e = step(t, set_of(t, st), t->Ncur, t->segY + static_cast<size_t>(st - s0) * 4 * un, s);
        for (int st = s1 - 1; st >= s0 && e == cudaSuccess; --st) {
            const int m = set_of(t, st);
            const double* Ys = t->segY + static_cast<size_t>(st - s0) * 4 * un;
            e = cudaMemcpyAsync(lsum, lam, sizeof(double) * un, cudaMemcpyDeviceToDevice, s);
            for (int q = 3; q >= 0 && e == cudaSuccess; --q) {
                const double w = (q == 0 || q == 3) ? c6 : 2.0 * c6;
                adj_coeff_kernel<<<blocks(t->n), 256, 0, s>>>(t->a, lam, t->mu, w,
                                                              q < 3 ? cs[q] : 0.0, t->n, q == 3);
                e = cudaGetLastError();
                if (e == cudaSuccess) e = vjp(t, m, Ys + q * un, g_agg, g_brk, s);
                if (e == cudaSuccess) {
                    adj_sum_kernel<<<blocks(t->n), 256, 0, s>>>(lsum, t->mu, t->n);
                    e = cudaGetLastError();
                }
            }
            std::swap(lam, lsum);
        }
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(gN0, lam, sizeof(double) * un, cudaMemcpyDeviceToDevice, s);
    return e;
}

// Captures `enqueue` on the tape's capture stream into *exec (replacing an
// older graph), instantiates it and moves it to the device.
template <class Fn>
cudaError_t capture(pbe_rk4_tape* t, cudaGraphExec_t* exec, Fn&& enqueue)
{
    if (*exec) { cudaGraphExecDestroy(*exec); *exec = nullptr; }
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(t->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    const cudaError_t le = enqueue(t->cap);
    e = cudaStreamEndCapture(t->cap, &graph);
    if (le != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return le; }
    if (e != cudaSuccess) return e;
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { *exec = nullptr; return e; }
    e = cudaGraphUpload(*exec, t->cap);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->cap);
    return e;
}

bool same_key(const double* const* key, const pbe_rk4_tape* t)
{
    return key[0] == t->x && key[1] == t->t_q && key[2] == t->bw_q;
}

cudaError_t forward(pbe_rk4_tape* t, double* N, cudaStream_t s)
{
    if (!t->use_graphs) return enqueue_forward(t, N, s);
    const size_t bytes = sizeof(double) * static_cast<size_t>(t->n);
    cudaError_t e = cudaSuccess;
    if (!t->fwd_exec || !same_key(t->fwd_key, t)) {
        e = capture(t, &t->fwd_exec, [&](cudaStream_t c) { return enqueue_forward(t, t->Nio, c); });
        if (e != cudaSuccess) return e;
        t->fwd_key[0] = t->x; t->fwd_key[1] = t->t_q; t->fwd_key[2] = t->bw_q;
    }
    e = cudaMemcpyAsync(t->Nio, N, bytes, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaGraphLaunch(t->fwd_exec, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(N, t->Nio, bytes, cudaMemcpyDeviceToDevice, s);
    return e;
}

cudaError_t backward(pbe_rk4_tape* t, const double* lamT, double* gN0, double* g_agg,
                     double* g_brk, cudaStream_t s)
{
    if (!t->use_graphs) return enqueue_backward(t, lamT, gN0, g_agg, g_brk, s);
    const size_t bytes = sizeof(double) * static_cast<size_t>(t->n);
    double* ga = t->g_int;
    double* gb = t->g_int + 3 * t->n_sets;
    cudaError_t e = cudaSuccess;
    if (!t->bwd_exec || !same_key(t->bwd_key, t)) {
        e = capture(t, &t->bwd_exec, [&](cudaStream_t c) {
            return enqueue_backward(t, t->lam_in, t->gN_out, ga, gb, c);
        });
        if (e != cudaSuccess) return e;
        t->bwd_key[0] = t->x; t->bwd_key[1] = t->t_q; t->bwd_key[2] = t->bw_q;
    }
    e = cudaMemcpyAsync(t->lam_in, lamT, bytes, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaGraphLaunch(t->bwd_exec, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(gN0, t->gN_out, bytes, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && t->kernel >= 0)
        e = cudaMemcpyAsync(g_agg, ga, sizeof(double) * 3 * t->n_sets, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && t->selection >= 0)
        e = cudaMemcpyAsync(g_brk, gb, sizeof(double) * 4 * t->n_sets, cudaMemcpyDeviceToDevice, s);
    return e;
}

template <class T>
cudaError_t tape_alloc(pbe_rk4_tape* t, T** out, size_t bytes)
{
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(bytes, 256));
    if (e != cudaSuccess) return e;
    t->allocs.push_back(q);
    *out = static_cast<T*>(q);
    return cudaSuccess;
}

void destroy(pbe_rk4_tape* t)
{
    if (t->fwd_exec) cudaGraphExecDestroy(t->fwd_exec);
    if (t->bwd_exec) cudaGraphExecDestroy(t->bwd_exec);
    if (t->cap) cudaStreamDestroy(t->cap);
    for (void* q : t->allocs) cudaFree(q);
    delete t;
}

} // namespace
} // namespace pbe_gb300

using namespace pbe_gb300;

extern "C" {

int pbe_rk4_tape_create(pbe_rk4_tape_t* tape, int n_steps, double dt, int checkpoint_every,
                        int n_sets, const pbe_agg_params_t* agg_sets,
                        const pbe_brk_params_t* brk_sets, const int* step_set)
{
    if (!tape) return cudaErrorInvalidValue;
    *tape = nullptr;
    if (n_steps < 0 || checkpoint_every <= 0 || n_sets <= 0 || !std::isfinite(dt))
        return cudaErrorInvalidValue;
    if (!agg_sets && !brk_sets) return cudaErrorInvalidValue;
    const int n = agg_sets ? agg_sets[0].n : brk_sets[0].n;
    if (n <= 0) return cudaErrorInvalidValue;
    for (int m = 0; m < n_sets; ++m) {
        if (agg_sets && (agg_sets[m].n != n || agg_sets[m].kernel_type != agg_sets[0].kernel_type ||
                         agg_sets[m].kernel_type < 0 || agg_sets[m].kernel_type > 5))
            return cudaErrorInvalidValue;
        if (brk_sets && (brk_sets[m].n != n || brk_sets[m].selection != brk_sets[0].selection ||
                         brk_sets[m].n_quad != brk_sets[0].n_quad || brk_sets[m].n_quad <= 0 ||
                         brk_sets[m].selection < 0 || brk_sets[m].selection > 3))
            return cudaErrorInvalidValue;
    }
    if (brk_sets && static_cast<long long>(n) * brk_sets[0].n_quad > 0x7fffffffLL)
        return cudaErrorInvalidValue;
    if (step_set)
        for (int s = 0; s < n_steps; ++s)
            if (step_set[s] < 0 || step_set[s] >= n_sets) return cudaErrorInvalidValue;
    pbe_rk4_tape* t = new (std::nothrow) pbe_rk4_tape();
    if (!t) return cudaErrorMemoryAllocation;
    t->n = n;
    t->n_steps = n_steps;
    t->every = checkpoint_every;
    t->n_sets = n_sets;
    t->dt = dt;
    if (agg_sets) { t->agg.assign(agg_sets, agg_sets + n_sets); t->kernel = agg_sets[0].kernel_type; }
    if (brk_sets) {
        t->brk.assign(brk_sets, brk_sets + n_sets);
        t->selection = brk_sets[0].selection;
        t->nq = brk_sets[0].n_quad;
    }
    if (step_set) t->step_set.assign(step_set, step_set + n_steps);
    cudaError_t e = cudaGetDevice(&t->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&t->num_sms, cudaDevAttrMultiProcessorCount, t->device);
    const size_t dn = sizeof(double) * static_cast<size_t>(n);
    const int nck = std::max(1, (n_steps + checkpoint_every - 1) / checkpoint_every);
    const int seg = std::min(checkpoint_every, std::max(n_steps, 1));
    if (e == cudaSuccess) e = tape_alloc(t, &t->ckpt, dn * nck);
    if (e == cudaSuccess) e = tape_alloc(t, &t->segY, dn * 4 * seg);
    for (double** p : {&t->k, &t->acc, &t->Y, &t->Ncur, &t->lam, &t->lsum, &t->a, &t->mu,
                       &t->Nio, &t->lam_in, &t->gN_out})
        if (e == cudaSuccess) e = tape_alloc(t, p, dn);
    if (e == cudaSuccess) e = tape_alloc(t, &t->g_int, sizeof(double) * 7 * n_sets);
    if (const char* g = std::getenv("PBE_GB300_TAPE_GRAPH")) t->use_graphs = std::strcmp(g, "0") != 0;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&t->cap, cudaStreamNonBlocking);
    for (int m = 0; m < n_sets && e == cudaSuccess; ++m) {
        void* w = nullptr;
        if (t->kernel >= 0) {
            e = tape_alloc(t, &w, agg_ws_layout(n, nullptr, nullptr));
            t->agg_ws.push_back(w);
        }
        if (e == cudaSuccess && t->selection >= 0) {
            e = tape_alloc(t, &w, brk_ws_layout(n, t->nq, nullptr, nullptr));
            t->brk_ws.push_back(w);
        }
    }
    if (e == cudaSuccess) e = tape_alloc(t, &t->vjp_ws, vjp_ws_layout(n, nullptr, nullptr));
    if (e != cudaSuccess) { destroy(t); return e; }
    *tape = t;
    return cudaSuccess;
}

int pbe_rk4_tape_destroy(pbe_rk4_tape_t tape)
{
    if (tape) destroy(tape);
    return cudaSuccess;
}

int pbe_rk4_tape_forward(pbe_rk4_tape_t tape, double* N, const double* x, const double* t_q,
                         const double* bw_q, void* stream)
{
    if (!tape) return cudaErrorInvalidValue;
    if (!N || !x || (tape->selection >= 0 && (!t_q || !bw_q))) return cudaErrorInvalidDevicePointer;
    tape->x = x;
    tape->t_q = t_q;
    tape->bw_q = bw_q;
    const cudaError_t e = forward(tape, N, static_cast<cudaStream_t>(stream));
    tape->recorded = (e == cudaSuccess);
    return e;
}

int pbe_rk4_tape_backward(pbe_rk4_tape_t tape, const double* lambda_T, double* gN0,
                          double* g_agg, double* g_brk, void* stream)
{
    if (!tape) return cudaErrorInvalidValue;
    if (!tape->recorded) return cudaErrorInvalidValue;
    if (!lambda_T || !gN0 || (tape->kernel >= 0 && !g_agg) || (tape->selection >= 0 && !g_brk))
        return cudaErrorInvalidDevicePointer;
    return backward(tape, lambda_T, gN0, g_agg, g_brk, static_cast<cudaStream_t>(stream));
}

} // extern "C"
