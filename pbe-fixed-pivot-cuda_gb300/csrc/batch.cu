// =============================================================================
// batch.cu -- host side of the batched-cell path: plans, the task scheduler,
// the tile-group autotuner, RK4 as one CUDA graph, the per-cell launch loop,
// and the pbe_batch_* C ABI (include/pbe_gb300.h).
//
// Schedule. Every cell is cut into tiles of kTileW bins; a tile task costs
// about min(I + W, n) lags. Cells are classed by floor(log2 n). Each class has a group
// size T (threads per task): a bundle packs 256/T tasks of one class, so a
// CTA of the persistent kernel runs up to eight small tiles at once. Bundles
// are sorted by work (largest first) and pulled from an atomic counter. A
// plan with few tiles (a handful of cells) also cuts each tile's lags into
// chunks (chunk_setup) and gathers the breakage term in the pair tasks
// instead of one prep CTA per cell; its VJP takes larger groups.
//
// Per call. The selection function of every bin is evaluated once per call
// into the plan's cache (sel_cache, SelScope). The adaptive integrators and
// the GMRES solves pass a per-cell skip mask, so finished cells and ended
// solves are left out of the prep and pair launches.
//
// Autotuner. With PBE_BATCH_TUNE, each class present in the plan times the
// persistent kernel on its own tasks for T = 32, 64, 128, 256 (synthetic
// state; the work of a tile does not depend on the values) and keeps the
// fastest. Results are cached per process and device (key: SM count, kernel
// type, breakage on/off, class) and, when PBE_GB300_TUNE_CACHE names a file,
// in that file (one "sms kernel brk class T" line per entry).
//
// RK4. A step is four (prep, main) launch pairs; the prep of a stage applies
// the previous stage's update in place (batch_internal.cuh, BatchStage).
// pbe_batch_rk4 captures n_steps steps plus the closing update into one CUDA
// graph on a private stream and launches it on the caller's stream.
//
// Beyond RK4: embedded Dormand-Prince 5(4) with a step size per cell
// (pbe_batch_rk45), Jacobian-vector products (pbe_batch_jvp), and the
// linearly implicit ROS2 (pbe_batch_ros2, pbe_batch_ros2_adaptive), whose
// stage systems are solved by matrix-free, right-preconditioned GMRES(m)
// with an optional tolerance and restarts (batch_implicit.cu).
// =============================================================================
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "batch_internal.cuh"

struct pbe_batch_plan {
    int device = 0;
    int num_sms = 0;
    int n_grids = 0, n_cells = 0, kernel = -1, selection = -1, nq = 0;
    long long total = 0;
    int max_n = 0;
    std::vector<int> grid_n, grid_off, cell_n, cell_grid;
    std::vector<long long> offsets;
    pbe_gb300::BatchDev d{};
    std::vector<void*> allocs;
    int group_size[16] = {0};
    int4* d_bundles = nullptr;
    int4* d_tasks = nullptr;
    std::vector<char> grid_geo;        // grids verified geometric (lag chunks apply)
    std::vector<double> t_q, bw_q;
    double* d_tq = nullptr;
    double* d_bw = nullptr;
    // death-GEMM work items (built on first use)
    int4* d_death_items = nullptr;
    int* d_gcells = nullptr;
    int n_death_items = -1;
    int death_split = 1;               // k slices of the death GEMM
    double* death_part = nullptr;      // [death_split * total] slice partials
    double* death_b = nullptr;         // every used grid's B matrix (death GEMM)
    long long* death_boff = nullptr;   // [n_grids] its offsets (device)
    // batched VJP (set up on first use)
    bool vjp_ready = false;
    pbe_gb300::BatchVjpDev vd{};
    // batched RK4 tape (allocated on first use, grown as needed)
    double* t_ckpt = nullptr;
    double* t_segY = nullptr;
    double* t_work = nullptr;          // tN, lam, lsum, a, mu
    size_t t_ckpt_cap = 0, t_seg_cap = 0;
    bool t_recorded = false;
    int t_steps = 0, t_every = 1;
    double t_dt = 0.0;
    const pbe_batch_cell_params_t* t_params = nullptr;
    // embedded RK 5(4) state (allocated on first use)
    double* rk_k = nullptr;            // 7 packed stage derivatives
    double* rk_cell = nullptr;         // t, dt per cell
    int* rk_int = nullptr;             // status, steps, rejects per cell; done counter
    // linearly implicit (Rosenbrock) integrator: GMRES state and stage vectors
    pbe_gb300::GmresDev gm{};
    int gm_cap = 0;                    // Krylov dimension the GMRES buffers hold
    double krylov_tol = 0.0;           // relative residual that ends a solve early (0: never)
    int krylov_restarts = 0;           // further GMRES cycles for cells above krylov_tol
    double* ros = nullptr;             // F, K1, K2, Y (4 packed vectors)
    double* ros_cell = nullptr;        // adaptive: t, dt, gamma dt per cell
    int* ros_int = nullptr;            // adaptive: status, steps, rejects per cell; done
    // selection function per cell bin for one multi-stage call (sel_cache);
    // allocated with the plan, so that a call under stream capture allocates nothing
    double* sx = nullptr;
    // per-cell launch loop scratch (allocated on first use)
    void* cell_agg_ws = nullptr;
    void* cell_brk_ws = nullptr;
    // graph cache
    cudaStream_t cap = nullptr;
    cudaGraphExec_t exec = nullptr;
    const void* g_N = nullptr;
    const void* g_params = nullptr;
    double g_dt = 0.0;
    int g_steps = 0;
};

namespace pbe_gb300 {
namespace {

constexpr int W = kTileW;
constexpr int kClasses = 16;

int n_class(int n)
{
    int c = 0;
    while ((2 << c) <= n && c < kClasses - 1) ++c;
    return c;
}

// Default group size per class (what the autotuner picked on GB300 for the
// 4096-cell workload: the reduction of 2 (W+1) T partial sums per task costs
// more than the lanes a small group leaves idle), 128 for very large cells.
int rule_group_size(int cls)
{
    if (cls <= 7) return 64;      // n < 256
    if (cls <= 13) return 32;     // n < 16384
    return 128;
}

// ---- tune cache ----------------------------------------------------------------
using TuneKey = std::tuple<int, int, int, int>;   // sms, kernel, brk, class
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune;
bool g_tune_file_read = false;

const char* tune_file() { return std::getenv("PBE_GB300_TUNE_CACHE"); }

void tune_cache_load_locked()
{
    if (g_tune_file_read) return;
    g_tune_file_read = true;
    const char* path = tune_file();
    if (!path || !*path) return;
    FILE* f = std::fopen(path, "r");
    if (!f) return;
    int a, b, c, e, t;
    while (std::fscanf(f, "%d %d %d %d %d", &a, &b, &c, &e, &t) == 5)
        if (t == 32 || t == 64 || t == 128 || t == 256) g_tune[TuneKey(a, b, c, e)] = t;
    std::fclose(f);
}

void tune_cache_store_locked(const TuneKey& k, int t)
{
    g_tune[k] = t;
    const char* path = tune_file();
    if (!path || !*path) return;
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%d %d %d %d %d\n", std::get<0>(k), std::get<1>(k), std::get<2>(k),
                 std::get<3>(k), t);
    std::fclose(f);
}

// ---- schedule ------------------------------------------------------------------
struct HostTask { int cell, I, chunk, nct; long long cost; };

long long task_cost(int n, int I, int T)
{
    const long long lags = std::min(I + W, n);
    const long long it = (lags + T - 1) / T;
    return it * T + 4LL * T;                          // + reduction / epilogue
}

// Bundles for the cells of the classes selected by `want` (all when null),
// each class with its group size gs[class]; sorted by work, largest first.
// vjp: row tiles of the VJP, whose work does not depend on the first row (every
// row meets all n partners).
void build_schedule(const pbe_batch_plan& p, const int* gs, const bool* want,
                    std::vector<int4>& bundles, std::vector<int4>& tasks, bool vjp = false)
{
    std::vector<std::vector<HostTask>> per(kClasses);
    const int Cg = p.d.Cg;
    for (int c = 0; c < p.n_cells; ++c) {
        const int n = p.cell_n[c];
        const int cls = n_class(n);
        if (want && !want[cls]) continue;
        if (vjp) {
            for (int I = 0; I < n; I += W) per[cls].push_back({c, I, 0, 1, task_cost(n, n, gs[cls])});
        } else {
            // forward tiles aligned to the top: the lowest may start below bin 0;
            // tile t spans the lags below n - W t, cut into chunks of Cg lags
            // when the plan has few tiles (chunk_setup)
            const bool chunks = Cg > 0 && p.grid_geo[p.cell_grid[c]];
            for (int I = n - W; I > -W; I -= W) {
                const int span = I + W;
                const int nct = chunks ? (span + Cg - 1) / Cg : 1;
                for (int k = 0; k < nct; ++k) {
                    const int lags = nct > 1 ? std::min(Cg, span - k * Cg) : span;
                    per[cls].push_back({c, I, k, nct, task_cost(n, lags - W, gs[cls])});
                }
            }
        }
    }
    struct B { long long cost; int cls; int first; int cnt; };
    std::vector<B> bl;
    std::vector<std::vector<HostTask>> sorted(kClasses);
    for (int cls = 0; cls < kClasses; ++cls) {
        auto& v = per[cls];
        if (v.empty()) continue;
        std::stable_sort(v.begin(), v.end(),
                         [](const HostTask& a, const HostTask& b) { return a.cost > b.cost; });
        const int per_b = kMainThreads / gs[cls];
        for (size_t i = 0; i < v.size(); i += per_b) {
            const int cnt = static_cast<int>(std::min<size_t>(per_b, v.size() - i));
            long long cost = 0;
            for (int k = 0; k < cnt; ++k) cost += v[i + k].cost;
            bl.push_back({cost, cls, static_cast<int>(i), cnt});
        }
        sorted[cls] = v;
    }
    std::stable_sort(bl.begin(), bl.end(), [](const B& a, const B& b) { return a.cost > b.cost; });
    bundles.clear();
    tasks.clear();
    for (const B& b : bl) {
        bundles.push_back(make_int4(static_cast<int>(tasks.size()), b.cnt, gs[b.cls], 0));
        for (int k = 0; k < b.cnt; ++k) {
            const HostTask& t = sorted[b.cls][b.first + k];
            tasks.push_back(make_int4(t.cell, t.I, t.chunk, t.nct));
        }
    }
}

template <class T>
cudaError_t plan_alloc(pbe_batch_plan* p, T** out, size_t count)
{
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    p->allocs.push_back(q);
    *out = static_cast<T*>(q);
    return cudaSuccess;
}

cudaError_t upload_schedule(pbe_batch_plan* p, const std::vector<int4>& b,
                            const std::vector<int4>& t, int4** db, int4** dt, cudaStream_t s)
{
    cudaError_t e = plan_alloc(p, db, b.size());
    if (e == cudaSuccess) e = plan_alloc(p, dt, t.size());
    if (e == cudaSuccess && !b.empty())
        e = cudaMemcpyAsync(*db, b.data(), b.size() * sizeof(int4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !t.empty())
        e = cudaMemcpyAsync(*dt, t.data(), t.size() * sizeof(int4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
}

void free_last(pbe_batch_plan* p, int count)
{
    for (int i = 0; i < count && !p->allocs.empty(); ++i) {
        cudaFree(p->allocs.back());
        p->allocs.pop_back();
    }
}

// Times the persistent kernel on the tasks of one class for each group size.
cudaError_t tune_class(pbe_batch_plan* p, int cls, const pbe_batch_cell_params_t* dparams,
                       double* dN, double* dout, cudaStream_t s, int* best_T)
{
    static const int cand[4] = {32, 64, 128, 256};
    bool want[kClasses] = {false};
    want[cls] = true;
    float best = 0.0f;
    *best_T = rule_group_size(cls);
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e != cudaSuccess) return e;
    e = cudaEventCreate(&e1);
    if (e != cudaSuccess) { cudaEventDestroy(e0); return e; }
    for (int ci = 0; ci < 4 && e == cudaSuccess; ++ci) {
        int gs[kClasses];
        for (int c = 0; c < kClasses; ++c) gs[c] = cand[ci];
        std::vector<int4> b;
        std::vector<int4> t;
        build_schedule(*p, gs, want, b, t);
        int4* db = nullptr;
        int4* dt = nullptr;
        e = upload_schedule(p, b, t, &db, &dt, s);
        if (e != cudaSuccess) break;
        const int nb = static_cast<int>(b.size());
        e = batch_main_bundles(p->d, dN, dparams, dout, false, db, dt, nb, s);   // warm-up
        if (e == cudaSuccess) e = cudaEventRecord(e0, s);
        for (int r = 0; r < 3 && e == cudaSuccess; ++r)
            e = batch_main_bundles(p->d, dN, dparams, dout, false, db, dt, nb, s);
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        free_last(p, 2);
        if (e == cudaSuccess && (ci == 0 || ms < best)) { best = ms; *best_T = cand[ci]; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return e;
}

cudaError_t autotune(pbe_batch_plan* p, bool retune, cudaStream_t s)
{
    bool present[kClasses] = {false};
    for (int c = 0; c < p->n_cells; ++c) present[n_class(p->cell_n[c])] = true;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    tune_cache_load_locked();
    // synthetic state and coefficients (any finite values: the work is value-independent)
    double* dN = nullptr;
    double* dout = nullptr;
    pbe_batch_cell_params_t* dparams = nullptr;
    const size_t np = static_cast<size_t>(p->total);
    cudaError_t e = plan_alloc(p, &dN, np);
    if (e == cudaSuccess) e = plan_alloc(p, &dout, np);
    if (e == cudaSuccess) e = plan_alloc(p, &dparams, static_cast<size_t>(p->n_cells));
    if (e != cudaSuccess) return e;
    {
        std::vector<double> ones(np, 1.0);
        std::vector<pbe_batch_cell_params_t> prm(static_cast<size_t>(p->n_cells));
        for (auto& q : prm) q = pbe_batch_cell_params_t{1e-15, 1e-17, 1.0, 1e-3, 1.0, 1.0, 0.0, 0.0};
        e = cudaMemcpyAsync(dN, ones.data(), np * sizeof(double), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dparams, prm.data(), prm.size() * sizeof(pbe_batch_cell_params_t),
                                cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = batch_prep(p->d, dN, dparams, kStageRhs, 0.0, 0.0, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    for (int cls = 0; cls < kClasses && e == cudaSuccess; ++cls) {
        if (!present[cls]) continue;
        const TuneKey key(p->num_sms, p->kernel, (p->nq > 0 ? 1 : 0) | (p->d.Cg > 0 ? 2 : 0), cls);
        auto it = g_tune.find(key);
        if (!retune && it != g_tune.end()) { p->group_size[cls] = it->second; continue; }
        int T = rule_group_size(cls);
        e = tune_class(p, cls, dparams, dN, dout, s, &T);
        if (e == cudaSuccess) {
            p->group_size[cls] = T;
            tune_cache_store_locked(key, T);
        }
    }
    free_last(p, 3);
    return e;
}

// Plans with few tiles (a handful of small cells) cut each tile of a cell on a
// geometric grid into chunks of Cg lags, about kChunkTasks tasks per CTA slot
// in all; the tile's last chunk task adds the chunk sums in chunk order and runs
// the epilogue. Cg is fixed for the plan, so a tile has the same chunks in every
// schedule built from it (tuning, class subsets, the Jacobian-vector pass).
cudaError_t chunk_setup(pbe_batch_plan* p, long long tiles, cudaStream_t s)
{
    BatchDev& d = p->d;
    d.Cg = 0;
    d.cbound = 1;
    std::vector<BatchGridDev> hg(static_cast<size_t>(p->n_grids));
    cudaError_t e = cudaMemcpyAsync(hg.data(), d.grids, hg.size() * sizeof(BatchGridDev),
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    p->grid_geo.assign(static_cast<size_t>(p->n_grids), 0);
    for (int g = 0; g < p->n_grids; ++g) p->grid_geo[g] = hg[g].geo != 0;
    if (p->kernel < 0 || tiles >= 4LL * 2 * p->num_sms) return cudaSuccess;
    long long lags = 0;
    int max_geo_n = 0;
    for (int c = 0; c < p->n_cells; ++c) {
        if (!p->grid_geo[p->cell_grid[c]]) continue;
        const long long n = p->cell_n[c], nt = (n + W - 1) / W;
        lags += nt * n - static_cast<long long>(W) * nt * (nt - 1) / 2;
        max_geo_n = std::max(max_geo_n, p->cell_n[c]);
    }
    if (lags == 0) return cudaSuccess;
    const long long target = static_cast<long long>(kChunkTasks) * 2 *
                             std::min(p->num_sms, kChunkMaxSms);
    long long cg = (lags + target - 1) / target;
    cg = std::max<long long>(((cg + 31) / 32) * 32, kChunkMinLags);
    if (cg >= max_geo_n) return cudaSuccess;
    const int Cg = static_cast<int>(cg);
    const int cbound = (max_geo_n + Cg - 1) / Cg;      // the top tile spans n lags
    const size_t nt = static_cast<size_t>(tiles);
    e = plan_alloc(p, &d.cpart, nt * static_cast<size_t>(cbound) * 2 * W);
    if (e == cudaSuccess) e = plan_alloc(p, &d.cticket, nt);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.cticket, 0, nt * sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    d.Cg = Cg;
    d.cbound = cbound;
    return cudaSuccess;
}

cudaError_t validate(int n_grids, const int* grid_n, const double* grid_x, int n_cells,
                     const int* cell_n, const int* cell_grid, int kernel, int selection,
                     int n_quad, const double* t_q, const double* bw_q)
{
    if (n_grids <= 0 || n_cells <= 0 || !grid_n || !grid_x || !cell_n || !cell_grid)
        return cudaErrorInvalidValue;
    if (kernel < -1 || kernel > 5 || selection < -1 || selection > 3) return cudaErrorInvalidValue;
    if (kernel < 0 && selection < 0) return cudaErrorInvalidValue;
    if (selection >= 0 && (n_quad <= 0 || !t_q || !bw_q)) return cudaErrorInvalidValue;
    if (selection < 0 && n_quad != 0) return cudaErrorInvalidValue;
    long long gtot = 0;
    for (int g = 0; g < n_grids; ++g) {
        if (grid_n[g] <= 0) return cudaErrorInvalidValue;
        const double* x = grid_x + gtot;
        for (int i = 0; i < grid_n[g]; ++i) {
            if (!(x[i] > 0.0) || !std::isfinite(x[i]) || !std::isnormal(x[i]))
                return cudaErrorInvalidValue;
            if (i > 0 && !(x[i] > x[i - 1])) return cudaErrorInvalidValue;
        }
        gtot += grid_n[g];
        // packed grid tables (n_quad (n + 2) run starts per grid) are int-indexed
        if ((gtot + 2LL * (g + 1)) * std::max(n_quad, 1) > 0x7fffffffLL) return cudaErrorInvalidValue;
    }
    long long ctot = 0;
    for (int c = 0; c < n_cells; ++c) {
        if (cell_grid[c] < 0 || cell_grid[c] >= n_grids) return cudaErrorInvalidValue;
        if (cell_n[c] <= 0 || cell_n[c] > grid_n[cell_grid[c]]) return cudaErrorInvalidValue;
        ctot += cell_n[c];
    }
    if (ctot > 0x7fffffffLL) return cudaErrorInvalidValue;
    for (int q = 0; q < n_quad; ++q)
        if (!(t_q[q] > 0.0 && t_q[q] <= 1.0) || !std::isfinite(bw_q[q])) return cudaErrorInvalidValue;
    return cudaSuccess;
}

cudaError_t create(pbe_batch_plan* p, int n_grids, const int* grid_n, const double* grid_x,
                   int n_cells, const int* cell_n, const int* cell_grid, int kernel,
                   int selection, int n_quad, const double* t_q, const double* bw_q, int flags,
                   cudaStream_t s)
{
    cudaError_t e = cudaGetDevice(&p->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, p->device);
    if (e != cudaSuccess) return e;
    p->n_grids = n_grids; p->n_cells = n_cells; p->kernel = kernel; p->selection = selection;
    p->nq = selection >= 0 ? n_quad : 0;
    p->grid_n.assign(grid_n, grid_n + n_grids);
    p->cell_n.assign(cell_n, cell_n + n_cells);
    p->cell_grid.assign(cell_grid, cell_grid + n_cells);
    std::vector<BatchGridDev> hg(static_cast<size_t>(n_grids));
    int goff = 0, foff = 0, woff = 0;
    p->grid_off.resize(static_cast<size_t>(n_grids));
    for (int g = 0; g < n_grids; ++g) {
        hg[g] = BatchGridDev{goff, grid_n[g], 0, 0, foff, woff, 0, 0};
        p->grid_off[g] = goff;
        goff += grid_n[g];
        foff += p->nq * (grid_n[g] + 2);
        woff += p->nq * grid_n[g];
    }
    std::vector<BatchCellDev> hc(static_cast<size_t>(n_cells));
    p->offsets.resize(static_cast<size_t>(n_cells) + 1);
    long long off = 0;
    long long tiles = 0;
    for (int c = 0; c < n_cells; ++c) {
        hc[c] = BatchCellDev{static_cast<int>(off), cell_n[c], cell_grid[c],
                             static_cast<int>(tiles)};
        p->offsets[c] = off;
        off += cell_n[c];
        tiles += (cell_n[c] + W - 1) / W;
        p->max_n = std::max(p->max_n, cell_n[c]);
    }
    p->offsets[n_cells] = off;
    p->total = off;

    BatchDev& d = p->d;
    d.n_grids = n_grids; d.n_cells = n_cells; d.kernel = kernel; d.selection = selection;
    d.nq = p->nq; d.num_sms = p->num_sms;
    // breakage gather in the pair tasks for plans of at most one wave of prep
    // CTAs (measured: one n = 3840 cell 358 -> 233 us per RHS, 64 cells
    // 1540 -> 1435 us; 1024 cells 20.84 -> 21.12 ms, so those keep the prep)
    bool tasks = p->nq > 0 && n_cells <= 2 * p->num_sms;
    if (flags & PBE_BATCH_BRK_PREP) tasks = false;
    if ((flags & PBE_BATCH_BRK_TASKS) && p->nq > 0) tasks = true;
    d.brk = tasks ? kBrkTasks : 0;
    const size_t G = static_cast<size_t>(goff), C = static_cast<size_t>(off);
    BatchCellDev* dcells = nullptr;
    e = plan_alloc(p, &d.grids, static_cast<size_t>(n_grids));
    if (e == cudaSuccess) e = plan_alloc(p, &dcells, static_cast<size_t>(n_cells));
    if (e == cudaSuccess) e = plan_alloc(p, &d.gx, G);
    if (e == cudaSuccess) e = plan_alloc(p, &d.ga, G);
    if (e == cudaSuccess) e = plan_alloc(p, &d.gia, G);
    if (e == cudaSuccess) e = plan_alloc(p, &d.ginv_dx, G);
    if (e == cudaSuccess) e = plan_alloc(p, &d.gBd, G);
    if (e == cudaSuccess) e = plan_alloc(p, &d.gSd, G);
    if (e == cudaSuccess) e = plan_alloc(p, &d.gLd, G);
    if (e == cudaSuccess) e = plan_alloc(p, &d.gSl, G);
    if (e == cudaSuccess) e = plan_alloc(p, &d.bfirst, static_cast<size_t>(foff));
    if (e == cudaSuccess) e = plan_alloc(p, &d.bwlo, static_cast<size_t>(woff));
    if (e == cudaSuccess) e = plan_alloc(p, &d.bwhi, static_cast<size_t>(woff));
    if (e == cudaSuccess) e = plan_alloc(p, &d.blo, static_cast<size_t>(woff));
    if (e == cudaSuccess) e = plan_alloc(p, &d.Y, C);
    if (e == cudaSuccess) e = plan_alloc(p, &d.Nj, C);
    if (e == cudaSuccess) e = plan_alloc(p, &d.Hj, C);
    if (e == cudaSuccess) e = plan_alloc(p, &d.Hk, C);
    if (e == cudaSuccess) e = plan_alloc(p, &d.SN, C);
    if (e == cudaSuccess) e = plan_alloc(p, &d.Bk, C);
    if (e == cudaSuccess) e = plan_alloc(p, &d.k, C);
    if (e == cudaSuccess) e = plan_alloc(p, &d.kacc, C);
    if (e == cudaSuccess) e = plan_alloc(p, &d.mom, static_cast<size_t>(n_cells) * 8);
    if (e == cudaSuccess) e = plan_alloc(p, &d.counter, 8);
    if (e == cudaSuccess) e = plan_alloc(p, &d.tfirst, static_cast<size_t>(tiles));
    if (e == cudaSuccess) e = plan_alloc(p, &d.tcarry, static_cast<size_t>(tiles));
    if (e == cudaSuccess) e = plan_alloc(p, &d.tticket, static_cast<size_t>(tiles));
    if (e == cudaSuccess && p->nq > 0) e = plan_alloc(p, &p->sx, C);
    if (e == cudaSuccess && p->nq > 0) e = plan_alloc(p, &p->d_tq, static_cast<size_t>(p->nq));
    if (e == cudaSuccess && p->nq > 0) e = plan_alloc(p, &p->d_bw, static_cast<size_t>(p->nq));
    if (e != cudaSuccess) return e;
    d.cells = dcells;
    // zero the stage arrays once: entries a kernel type never writes stay
    // finite for the loads that the tile body issues unconditionally
    for (double* a : {d.Y, d.Nj, d.Hj, d.Hk, d.SN, d.Bk, d.k, d.kacc})
        if (e == cudaSuccess) e = cudaMemsetAsync(a, 0, C * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.tticket, 0, static_cast<size_t>(tiles) * sizeof(int), s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d.grids, hg.data(), hg.size() * sizeof(BatchGridDev),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dcells, hc.data(), hc.size() * sizeof(BatchCellDev),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d.gx, grid_x, G * sizeof(double), cudaMemcpyHostToDevice, s);
    if (p->nq > 0) {
        p->t_q.assign(t_q, t_q + p->nq);
        p->bw_q.assign(bw_q, bw_q + p->nq);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p->d_tq, t_q, p->nq * sizeof(double), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p->d_bw, bw_q, p->nq * sizeof(double), cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess) e = batch_kernel_setup(kernel);
    if (e == cudaSuccess) e = batch_grid_tables(d, p->d_tq, p->d_bw, 0, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = chunk_setup(p, tiles, s);
    if (e != cudaSuccess) return e;

    // lag chunks: single-warp groups keep the fixed-order reduction (2 W T adds
    // per task) small next to a chunk's pairs
    for (int cls = 0; cls < kClasses; ++cls)
        p->group_size[cls] = d.Cg > 0 ? 32 : rule_group_size(cls);
    if (flags & (PBE_BATCH_TUNE | PBE_BATCH_RETUNE)) {
        e = autotune(p, (flags & PBE_BATCH_RETUNE) != 0, s);
        if (e != cudaSuccess) return e;
    }
    std::vector<int4> b;
    std::vector<int4> t;
    build_schedule(*p, p->group_size, nullptr, b, t);
    e = upload_schedule(p, b, t, &p->d_bundles, &p->d_tasks, s);
    if (e != cudaSuccess) return e;
    d.bundles = p->d_bundles;
    d.tasks = p->d_tasks;
    d.n_bundles = static_cast<int>(b.size());
    return cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
}

void destroy(pbe_batch_plan* p)
{
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->cap) cudaStreamDestroy(p->cap);
    for (void* q : p->allocs) cudaFree(q);
    delete p;
}

cudaError_t check_plan(pbe_batch_plan* p)
{
    if (!p) return cudaErrorInvalidValue;
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    return dev == p->device ? cudaSuccess : cudaErrorInvalidDevice;
}

// Selection function of every cell bin for the parameters of one call,
// computed once on s at the call's start by a kernel over all bins (for the
// power law one pow per bin instead of one per bin and stage, spread over
// every SM instead of one CTA per cell): the plan's kernels read it while the
// SelScope of the call is alive. Plans without breakage: nothing.
struct SelScope {
    pbe_batch_plan* p;
    explicit SelScope(pbe_batch_plan* q) : p(q) {}
    ~SelScope() { p->d.Sx = nullptr; }
    SelScope(const SelScope&) = delete;
    SelScope& operator=(const SelScope&) = delete;
};

cudaError_t sel_cache(pbe_batch_plan* p, const pbe_batch_cell_params_t* prm, cudaStream_t s)
{
    p->d.Sx = nullptr;
    if (p->selection < 0 || p->nq <= 0 || !p->sx) return cudaSuccess;
    cudaError_t e = batch_sel(p->d, prm, p->sx, p->total, s);   // (sx: allocated with the plan)
    if (e == cudaSuccess) p->d.Sx = p->sx;
    return e;
}

// One RK4 step sequence enqueued on s.
cudaError_t enqueue_rk4(pbe_batch_plan* p, double* N, const pbe_batch_cell_params_t* prm,
                        double dt, int n_steps, cudaStream_t s)
{
    SelScope scope(p);
    cudaError_t e0 = sel_cache(p, prm, s);
    if (e0 != cudaSuccess) return e0;
    const BatchDev& d = p->d;
    const double h = 0.5 * dt, dt6 = dt / 6.0;
    cudaError_t e = cudaSuccess;
    for (int step = 0; step < n_steps && e == cudaSuccess; ++step) {
        e = batch_prep(d, N, prm, step == 0 ? kStageRhs : kStageNext, 0.0, dt6, s);
        if (e == cudaSuccess) e = batch_main(d, N, prm, d.k, false, s);
        if (e == cudaSuccess) e = batch_prep(d, N, prm, kStageTwo, h, dt6, s);
        if (e == cudaSuccess) e = batch_main(d, d.Y, prm, d.k, false, s);
        if (e == cudaSuccess) e = batch_prep(d, N, prm, kStageThree, h, dt6, s);
        if (e == cudaSuccess) e = batch_main(d, d.Y, prm, d.k, false, s);
        if (e == cudaSuccess) e = batch_prep(d, N, prm, kStageThree, dt, dt6, s);
        if (e == cudaSuccess) e = batch_main(d, d.Y, prm, d.k, false, s);
    }
    if (e == cudaSuccess) e = batch_prep(d, N, prm, kStageFinish, 0.0, dt6, s);
    return e;
}

// Captures (if the cached graph does not match) without launching.
cudaError_t rk4_capture(pbe_batch_plan* p, double* N, const pbe_batch_cell_params_t* prm, double dt,
                        int n_steps)
{
    if (!p->exec || p->g_N != N || p->g_params != prm || p->g_dt != dt || p->g_steps != n_steps) {
        if (p->exec) { cudaGraphExecDestroy(p->exec); p->exec = nullptr; }
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        cudaError_t le = enqueue_rk4(p, N, prm, dt, n_steps, p->cap);
        e = cudaStreamEndCapture(p->cap, &graph);
        if (le != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return le; }
        if (e != cudaSuccess) return e;
        e = cudaGraphInstantiate(&p->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) { p->exec = nullptr; return e; }
        // move the executable graph to the device now, not at its first launch
        e = cudaGraphUpload(p->exec, p->cap);
        if (e == cudaSuccess) e = cudaStreamSynchronize(p->cap);
        if (e != cudaSuccess) return e;
        p->g_N = N; p->g_params = prm; p->g_dt = dt; p->g_steps = n_steps;
    }
    return cudaSuccess;
}

cudaError_t rk4_graph(pbe_batch_plan* p, double* N, const pbe_batch_cell_params_t* prm, double dt,
                      int n_steps, cudaStream_t s)
{
    cudaError_t e = rk4_capture(p, N, prm, dt, n_steps);
    if (e != cudaSuccess) return e;
    e = cudaGraphLaunch(p->exec, s);
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t rk4_percell(pbe_batch_plan* p, double* N, const pbe_batch_cell_params_t* prm,
                        double dt, int n_steps, cudaStream_t s)
{
    const BatchDev& d = p->d;
    if (!p->cell_agg_ws && p->kernel >= 0) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, agg_ws_layout(p->max_n, nullptr, nullptr));
        if (e != cudaSuccess) return e;
        p->allocs.push_back(q);
        p->cell_agg_ws = q;
    }
    if (!p->cell_brk_ws && p->nq > 0) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, brk_ws_layout(p->max_n, p->nq, nullptr, nullptr));
        if (e != cudaSuccess) return e;
        p->allocs.push_back(q);
        p->cell_brk_ws = q;
    }
    // the single-instance calls take their coefficients by value
    std::vector<pbe_batch_cell_params_t> hp(static_cast<size_t>(p->n_cells));
    cudaError_t e = cudaMemcpyAsync(hp.data(), prm, hp.size() * sizeof(pbe_batch_cell_params_t),
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    const double h = 0.5 * dt, dt6 = dt / 6.0;
    static const int kStages[4] = {kStageTwo, kStageThree, kStageThree, kStageFinish};
    const double cs[4] = {h, h, dt, 0.0};
    for (int step = 0; step < n_steps && e == cudaSuccess; ++step) {
        for (int c = 0; c < p->n_cells && e == cudaSuccess; ++c) {
            const int n = p->cell_n[c];
            const long long off = p->offsets[c];
            const double* x = d.gx + p->grid_off[p->cell_grid[c]];
            double* Nc = N + off;
            double* kc = d.k + off;
            double* ac = d.kacc + off;
            double* Yc = d.Y + off;
            const pbe_batch_cell_params_t& P = hp[c];
            for (int st = 0; st < 4 && e == cudaSuccess; ++st) {
                const double* in = (st == 0) ? Nc : Yc;
                e = cudaMemsetAsync(kc, 0, static_cast<size_t>(n) * sizeof(double), s);
                if (e == cudaSuccess && p->kernel >= 0) {
                    AggArgs a{in, x, kc, n, p->kernel, P.beta0, P.beta_br, P.beta_sh};
                    e = agg_launch(a, false, p->cell_agg_ws, p->num_sms, s);
                }
                if (e == cudaSuccess && p->nq > 0) {
                    BrkArgs b{in, x, p->d_tq, p->d_bw, kc, n, p->nq, p->selection,
                              P.S0, P.v_ref, P.alpha, P.v_min};
                    e = brk_launch(b, false, p->cell_brk_ws, s);
                }
                if (e == cudaSuccess) e = cell_stage(Nc, kc, ac, Yc, n, kStages[st], cs[st], dt6, s);
            }
        }
    }
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t vjp_setup(pbe_batch_plan* p, cudaStream_t s)
{
    if (p->vjp_ready) return cudaSuccess;
    BatchVjpDev& vd = p->vd;
    const size_t C = static_cast<size_t>(p->total);
    std::vector<int> tile_off(static_cast<size_t>(p->n_cells) + 1, 0);
    for (int c = 0; c < p->n_cells; ++c) tile_off[c + 1] = tile_off[c] + (p->cell_n[c] + W - 1) / W;
    // every row tile meets all n partners, so with few tiles larger groups
    // (fewer tasks per bundle) give each CTA slot a bundle: T >= 256 x (CTA
    // slots) / tiles, a power of two in [forward T, 256]
    int gs[kClasses];
    const long long tiles = tile_off.back();
    for (int c = 0; c < kClasses; ++c) {
        int T = p->group_size[c] > 0 ? p->group_size[c] : 32;
        while (T < kMainThreads && tiles * T < 256LL * 2 * p->num_sms) T <<= 1;
        gs[c] = T;
    }
    std::vector<int4> b;
    std::vector<int4> t;
    build_schedule(*p, gs, nullptr, b, t, true);
    int* dto = nullptr;
    int4* db = nullptr;
    int4* dt = nullptr;
    cudaError_t e = plan_alloc(p, &vd.h, C);
    if (e == cudaSuccess) e = plan_alloc(p, &vd.D, C);
    if (e == cudaSuccess) e = plan_alloc(p, &vd.mom, static_cast<size_t>(p->n_cells) * 16);
    if (e == cudaSuccess) e = plan_alloc(p, &vd.tpart, 2 * static_cast<size_t>(tile_off.back()));
    if (e == cudaSuccess) e = plan_alloc(p, &dto, tile_off.size());
    if (e == cudaSuccess) e = plan_alloc(p, &vd.counter, 8);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dto, tile_off.data(), tile_off.size() * sizeof(int),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = upload_schedule(p, b, t, &db, &dt, s);
    if (e == cudaSuccess) e = batch_vjp_setup(p->kernel);
    if (e != cudaSuccess) return e;
    vd.tile_off = dto;
    vd.bundles = db;
    vd.tasks = dt;
    vd.n_bundles = static_cast<int>(b.size());
    p->vjp_ready = true;
    return cudaSuccess;
}

// Batched RK4 steps [s0, s1) on N (the plan's stage machinery). first:
// stage 1 of step s0 evaluates at N as given (else it first closes the
// previous step). ckpt: N at every step multiple of `every` is copied to
// ckpt[step / every]. Ys: the stage states of every step are copied to
// Ys[((step - s0) * 4 + q) * total]. finish: close the last step.
// (The caller holds a SelScope with the selection of prm cached.)
cudaError_t run_steps(pbe_batch_plan* p, double* N, const pbe_batch_cell_params_t* prm, double dt,
                      int s0, int s1, bool first, double* ckpt, int every, double* Ys,
                      bool finish, cudaStream_t s)
{
    const BatchDev& d = p->d;
    const double h = 0.5 * dt, dt6 = dt / 6.0;
    const size_t C = static_cast<size_t>(p->total), bytes = C * sizeof(double);
    cudaError_t e = cudaSuccess;
    for (int st = s0; st < s1 && e == cudaSuccess; ++st) {
        double* Y = Ys ? Ys + static_cast<size_t>(st - s0) * 4 * C : nullptr;
        e = batch_prep(d, N, prm, (st == s0 && first) ? kStageRhs : kStageNext, 0.0, dt6, s);
        if (e == cudaSuccess && ckpt && st % every == 0)
            e = cudaMemcpyAsync(ckpt + static_cast<size_t>(st / every) * C, N, bytes,
                                cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess && Y) e = cudaMemcpyAsync(Y, N, bytes, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = batch_main(d, N, prm, d.k, false, s);
        const double cs[3] = {h, h, dt};
        for (int q = 1; q < 4 && e == cudaSuccess; ++q) {
            e = batch_prep(d, N, prm, q == 1 ? kStageTwo : kStageThree, cs[q - 1], dt6, s);
            if (e == cudaSuccess && Y)
                e = cudaMemcpyAsync(Y + q * C, d.Y, bytes, cudaMemcpyDeviceToDevice, s);
            if (e == cudaSuccess && (q < 3 || finish || st + 1 < s1))
                e = batch_main(d, d.Y, prm, d.k, false, s);
        }
    }
    if (e == cudaSuccess && finish) e = batch_prep(d, N, prm, kStageFinish, 0.0, dt6, s);
    return e;
}

cudaError_t tape_forward(pbe_batch_plan* p, double* N, const pbe_batch_cell_params_t* prm,
                         double dt, int n_steps, int every, cudaStream_t s)
{
    const size_t C = static_cast<size_t>(p->total);
    const size_t nck = static_cast<size_t>((n_steps + every - 1) / every);
    const size_t seg = static_cast<size_t>(std::min(every, n_steps));
    cudaError_t e = vjp_setup(p, s);
    if (e != cudaSuccess) return e;
    if (!p->t_work) {
        e = plan_alloc(p, &p->t_work, 5 * C);
        if (e != cudaSuccess) return e;
    }
    if (nck * C > p->t_ckpt_cap) {
        e = plan_alloc(p, &p->t_ckpt, nck * C);
        if (e != cudaSuccess) return e;
        p->t_ckpt_cap = nck * C;
    }
    if (4 * seg * C > p->t_seg_cap) {
        e = plan_alloc(p, &p->t_segY, 4 * seg * C);
        if (e != cudaSuccess) return e;
        p->t_seg_cap = 4 * seg * C;
    }
    p->t_recorded = false;
    SelScope scope(p);
    e = sel_cache(p, prm, s);
    if (e != cudaSuccess) return e;
    e = run_steps(p, N, prm, dt, 0, n_steps, true, p->t_ckpt, every, nullptr, true, s);
    if (e != cudaSuccess) return e;
    p->t_recorded = true;
    p->t_steps = n_steps;
    p->t_every = every;
    p->t_dt = dt;
    p->t_params = prm;
    return cudaSuccess;
}

cudaError_t tape_backward(pbe_batch_plan* p, const double* lamT, double* gN0, double* gp,
                          cudaStream_t s)
{
    const size_t C = static_cast<size_t>(p->total), bytes = C * sizeof(double);
    const long long nC = static_cast<long long>(C);
    double* tN = p->t_work;
    double* lam = p->t_work + C;
    double* lsum = p->t_work + 2 * C;
    double* a = p->t_work + 3 * C;
    double* mu = p->t_work + 4 * C;
    const double dt = p->t_dt, h = 0.5 * dt, c6 = dt / 6.0;
    const double cs[3] = {h, h, dt};
    const pbe_batch_cell_params_t* prm = p->t_params;
    SelScope scope(p);
    cudaError_t e = sel_cache(p, prm, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(lam, lamT, bytes, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(gp, 0, sizeof(double) * 8 * static_cast<size_t>(p->n_cells), s);
    const int every = p->t_every;
    const int nseg = (p->t_steps + every - 1) / every;
    for (int g = nseg - 1; g >= 0 && e == cudaSuccess; --g) {
        const int s0 = g * every, s1 = std::min(s0 + every, p->t_steps);
        e = cudaMemcpyAsync(tN, p->t_ckpt + static_cast<size_t>(g) * C, bytes,
                            cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess)
            e = run_steps(p, tN, prm, dt, s0, s1, true, nullptr, every, p->t_segY, false, s);
        for (int st = s1 - 1; st >= s0 && e == cudaSuccess; --st) {
            const double* Ys = p->t_segY + static_cast<size_t>(st - s0) * 4 * C;
            e = cudaMemcpyAsync(lsum, lam, bytes, cudaMemcpyDeviceToDevice, s);
            for (int q = 3; q >= 0 && e == cudaSuccess; --q) {
                const double w = (q == 0 || q == 3) ? c6 : 2.0 * c6;
                e = batch_adj_coeff(a, lam, mu, w, q < 3 ? cs[q] : 0.0, nC, q == 3, s);
                if (e == cudaSuccess) e = batch_vjp(p->d, p->vd, Ys + q * C, a, mu, gp, prm, s);
                if (e == cudaSuccess) e = batch_adj_sum(lsum, mu, nC, s);
            }
            std::swap(lam, lsum);
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(gN0, lam, bytes, cudaMemcpyDeviceToDevice, s);
    return e;
}

// Dormand-Prince 5(4) tableau (Dormand & Prince, J. Comput. Appl. Math. 6 (1980)):
// stage s (2..7) combines k_1 .. k_{s-1}; the 7th stage is the 5th-order
// solution (first-same-as-last); kErr = b5 - b4 weights the error estimate.
const double kDP[6][6] = {
    {1.0 / 5.0},
    {3.0 / 40.0, 9.0 / 40.0},
    {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0},
    {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0},
    {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0},
    {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0}};
const double kDPErr[7] = {71.0 / 57600.0, 0.0, -71.0 / 16695.0, 71.0 / 1920.0,
                          -17253.0 / 339200.0, 22.0 / 525.0, -1.0 / 40.0};

// ---- Jacobian-vector products and the Rosenbrock integrator -------------------
// J(N) v = T(N, v) + T(v, N) for the aggregation part (two passes of the pair
// kernel with the j side from the first vector, batch_kernels.cu) plus the
// breakage Jacobian at N applied to v (first pass).
// skip (device, n_cells, or null): cells left out of both passes (their
// out entries keep their old values).
cudaError_t jvp(pbe_batch_plan* p, const double* N, const double* v,
                const pbe_batch_cell_params_t* prm, double* out, cudaStream_t s,
                const int* skip = nullptr)
{
    if (!p->d.Ha) {
        cudaError_t e = plan_alloc(p, &p->d.Ha, static_cast<size_t>(p->total));
        if (e != cudaSuccess) { p->d.Ha = nullptr; return e; }
    }
    BatchDev d = p->d;
    d.skip = skip;
    BatchDev d1 = d;
    d1.A = N;
    cudaError_t e = batch_jvp_prep(d, N, v, N, prm, true, s);
    if (e == cudaSuccess) e = batch_main(d1, v, prm, out, false, s);
    BatchDev d2 = d;
    d2.A = v;
    d2.brk |= kBrkNone;                    // breakage is linear: first pass only
    if (e == cudaSuccess) e = batch_jvp_prep(d, v, N, N, prm, false, s);
    if (e == cudaSuccess) e = batch_main(d2, N, prm, out, true, s);
    return e;
}

cudaError_t gmres_alloc(pbe_batch_plan* p, int m)
{
    if (p->gm_cap >= m) return cudaSuccess;
    const size_t C = static_cast<size_t>(p->total), nc = static_cast<size_t>(p->n_cells);
    const size_t M = static_cast<size_t>(m);
    GmresDev g{};
    cudaError_t e = plan_alloc(p, &g.V, (M + 1) * C);
    if (e == cudaSuccess) e = plan_alloc(p, &g.Z, C);
    if (e == cudaSuccess) e = plan_alloc(p, &g.W, C);
    if (e == cudaSuccess) e = plan_alloc(p, &g.P, C);
    if (e == cudaSuccess) e = plan_alloc(p, &g.H, nc * (M + 1) * M);
    if (e == cudaSuccess) e = plan_alloc(p, &g.gv, nc * (M + 1));
    if (e == cudaSuccess) e = plan_alloc(p, &g.cs, nc * M);
    if (e == cudaSuccess) e = plan_alloc(p, &g.sn, nc * M);
    if (e == cudaSuccess) e = plan_alloc(p, &g.beta0, nc);
    if (e == cudaSuccess) e = plan_alloc(p, &g.kval, nc);
    if (e == cudaSuccess) e = plan_alloc(p, &g.done, nc);
    if (e == cudaSuccess) e = plan_alloc(p, &g.R, C);
    if (e == cudaSuccess) e = plan_alloc(p, &g.rnorm, nc);
    if (e == cudaSuccess) e = plan_alloc(p, &g.last, nc);
    if (e == cudaSuccess) e = plan_alloc(p, &g.conv, nc);
    if (e != cudaSuccess) return e;
    p->gm = g;
    p->gm_cap = m;
    return cudaSuccess;
}

// One GMRES cycle of every cell that needs it (gmres_solve).
cudaError_t gmres_cycle(pbe_batch_plan* p, const double* N, const double* r, double* x,
                        const pbe_batch_cell_params_t* prm, double* resid, bool first, bool final,
                        cudaStream_t s)
{
    const BatchDev& d = p->d;
    const GmresDev& g = p->gm;
    cudaError_t e = batch_gmres_start(d, g, N, r, prm, first, s);
    for (int j = 0; j < g.m && e == cudaSuccess; ++j) {
        // cells whose cycle has ended (or never started) are left out
        e = jvp(p, N, g.Z, prm, g.W, s, g.done);
        if (e == cudaSuccess) e = batch_gmres_arnoldi(d, g, j, s);
    }
    if (e == cudaSuccess) e = batch_gmres_finish(d, g, x, resid, !first, final, s);
    return e;
}

// x = (I - gt J(N))^-1 r for every cell: GMRES(m), right preconditioned
// (batch_implicit.cu), then up to g.restarts more cycles on r - A x for the
// cells above the tolerance (one Jacobian-vector product each to form the
// residual); resid[c] = max(resid[c], relative residual of the solve).
cudaError_t gmres_solve(pbe_batch_plan* p, const double* N, const double* r, double* x,
                        const pbe_batch_cell_params_t* prm, double* resid, cudaStream_t s)
{
    const GmresDev& g = p->gm;
    const int R = g.restarts;
    cudaError_t e = gmres_cycle(p, N, r, x, prm, resid, true, R == 0, s);
    for (int k = 1; k <= R && e == cudaSuccess; ++k) {
        e = jvp(p, N, x, prm, g.W, s, g.conv);
        if (e == cudaSuccess) e = batch_gmres_restart(p->d, g, r, x, s);
        if (e == cudaSuccess) e = gmres_cycle(p, N, g.R, x, prm, resid, false, k == R, s);
    }
    return e;
}

// ROS2 (two-stage, second order, L-stable; gamma = 1 + 1/sqrt 2):
//   (I - gamma dt J) k1 = R(N)
//   (I - gamma dt J) k2 = R(N + dt k1) - 2 k1
//   N += 3/2 dt k1 + 1/2 dt k2
// with J = J(N) for both stages, every cell of the plan at once.
cudaError_t ros2(pbe_batch_plan* p, double* N, const pbe_batch_cell_params_t* prm, double dt,
                 int n_steps, int m, double* resid, cudaStream_t s)
{
    const size_t C = static_cast<size_t>(p->total);
    cudaError_t e = gmres_alloc(p, m);
    if (e == cudaSuccess && !p->ros) {
        e = plan_alloc(p, &p->ros, 4 * C);
        if (e != cudaSuccess) p->ros = nullptr;
    }
    if (e != cudaSuccess) return e;
    p->gm.m = m;
    p->gm.total = static_cast<long long>(C);
    p->gm.gt = (1.0 + 1.0 / std::sqrt(2.0)) * dt;
    p->gm.gtc = nullptr;
    p->gm.skip = nullptr;
    p->gm.tol = p->krylov_tol;
    p->gm.restarts = p->krylov_restarts;
    SelScope scope(p);
    e = sel_cache(p, prm, s);
    if (e != cudaSuccess) return e;
    double* F = p->ros;
    double* K1 = p->ros + C;
    double* K2 = p->ros + 2 * C;
    double* Y = p->ros + 3 * C;
    const BatchDev& d = p->d;
    const long long T = static_cast<long long>(C);
    if (resid) e = cudaMemsetAsync(resid, 0, static_cast<size_t>(p->n_cells) * sizeof(double), s);
    for (int st = 0; st < n_steps && e == cudaSuccess; ++st) {
        e = batch_prep(d, N, prm, kStageRhs, 0.0, 0.0, s);
        if (e == cudaSuccess) e = batch_main(d, N, prm, F, false, s);
        if (e == cudaSuccess) e = gmres_solve(p, N, F, K1, prm, resid, s);
        if (e == cudaSuccess) e = batch_lincomb(Y, 1.0, N, dt, K1, T, p->num_sms, s);
        if (e == cudaSuccess) e = batch_prep(d, Y, prm, kStageRhs, 0.0, 0.0, s);
        if (e == cudaSuccess) e = batch_main(d, Y, prm, F, false, s);
        if (e == cudaSuccess) e = batch_lincomb(F, 1.0, F, -2.0, K1, T, p->num_sms, s);
        if (e == cudaSuccess) e = gmres_solve(p, N, F, K2, prm, resid, s);
        if (e == cudaSuccess) e = batch_ros_update(N, 1.5 * dt, K1, 0.5 * dt, K2, T, p->num_sms, s);
    }
    return e;
}

// ROS2 to t_end with a step size per cell (batch_implicit.cu: stage and
// controller kernels, Rk45Ctl conventions): attempts are enqueued in chunks of
// 4, then the count of finished cells is read back. A finished cell runs with
// dt = 0 and is left out of the RHS, Jacobian-vector and solve launches.
cudaError_t ros2_adaptive(pbe_batch_plan* p, double* N, const pbe_batch_cell_params_t* prm,
                          double t_end, double rtol, double atol, double dt0, int m,
                          int max_attempts, int* steps_out, int* rejects_out, int* attempts_out,
                          double* resid, cudaStream_t s)
{
    const size_t C = static_cast<size_t>(p->total), nc = static_cast<size_t>(p->n_cells);
    cudaError_t e = gmres_alloc(p, m);
    if (e == cudaSuccess && !p->ros) {
        e = plan_alloc(p, &p->ros, 4 * C);
        if (e != cudaSuccess) p->ros = nullptr;
    }
    if (e == cudaSuccess && !p->ros_cell) {
        e = plan_alloc(p, &p->ros_cell, 3 * nc);
        if (e == cudaSuccess) e = plan_alloc(p, &p->ros_int, 3 * nc + 1);
        if (e != cudaSuccess) { p->ros_cell = nullptr; p->ros_int = nullptr; }
    }
    if (e != cudaSuccess) return e;
    Rk45Ctl ctl;
    ctl.t = p->ros_cell;
    ctl.dt = p->ros_cell + nc;
    ctl.status = p->ros_int;
    ctl.steps = p->ros_int + nc;
    ctl.rejects = p->ros_int + 2 * nc;
    ctl.done = p->ros_int + 3 * nc;
    ctl.t_end = t_end;
    ctl.rtol = rtol;
    ctl.atol = atol;
    double* gtc = p->ros_cell + 2 * nc;
    p->gm.m = m;
    p->gm.total = static_cast<long long>(C);
    p->gm.gt = 0.0;
    p->gm.gtc = gtc;
    p->gm.skip = ctl.status;               // finished cells: no solve
    p->gm.tol = p->krylov_tol;
    p->gm.restarts = p->krylov_restarts;
    const double gamma = 1.0 + 1.0 / std::sqrt(2.0);
    std::vector<double> init(3 * nc, 0.0);
    for (size_t c = 0; c < nc; ++c) init[nc + c] = std::min(dt0, t_end);
    e = cudaMemcpyAsync(p->ros_cell, init.data(), init.size() * sizeof(double),
                        cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->ros_int, 0, (3 * nc + 1) * sizeof(int), s);
    if (e == cudaSuccess && resid) e = cudaMemsetAsync(resid, 0, nc * sizeof(double), s);
    SelScope scope(p);
    if (e == cudaSuccess) e = sel_cache(p, prm, s);
    if (e != cudaSuccess) return e;
    double* F = p->ros;
    double* K1 = p->ros + C;
    double* K2 = p->ros + 2 * C;
    double* Y = p->ros + 3 * C;
    BatchDev d = p->d;
    d.skip = ctl.status;                   // finished cells: no RHS work
    const long long T = static_cast<long long>(C);
    int attempts = 0, done = 0;
    while (e == cudaSuccess && attempts < max_attempts && done < p->n_cells) {
        const int chunk = std::min(4, max_attempts - attempts);
        for (int a = 0; a < chunk && e == cudaSuccess; ++a) {
            e = batch_ros2_stage(d, N, K1, Y, gtc, ctl, gamma, s);       // gamma dt per cell
            if (e == cudaSuccess) e = batch_prep(d, N, prm, kStageRhs, 0.0, 0.0, s);
            if (e == cudaSuccess) e = batch_main(d, N, prm, F, false, s);
            if (e == cudaSuccess) e = gmres_solve(p, N, F, K1, prm, resid, s);
            if (e == cudaSuccess) e = batch_ros2_stage(d, N, K1, Y, gtc, ctl, gamma, s);
            if (e == cudaSuccess) e = batch_prep(d, Y, prm, kStageRhs, 0.0, 0.0, s);
            if (e == cudaSuccess) e = batch_main(d, Y, prm, F, false, s);
            if (e == cudaSuccess) e = batch_lincomb(F, 1.0, F, -2.0, K1, T, p->num_sms, s);
            if (e == cudaSuccess) e = gmres_solve(p, N, F, K2, prm, resid, s);
            if (e == cudaSuccess) e = batch_ros2_control(d, N, K1, K2, ctl, s);
        }
        attempts += chunk;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&done, ctl.done, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    if (e == cudaSuccess && steps_out)
        e = cudaMemcpyAsync(steps_out, ctl.steps, nc * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && rejects_out)
        e = cudaMemcpyAsync(rejects_out, ctl.rejects, nc * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (attempts_out) *attempts_out = attempts;
    if (e != cudaSuccess) return e;
    return done == p->n_cells ? cudaSuccess : cudaErrorNotReady;
}

// Adaptive embedded RK 5(4) for every cell to t_end: attempts are enqueued
// in chunks of 8 (6 RHS evaluations and one control launch each), then the
// count of finished cells is read back. Finished cells are left out of the
// RHS launches.
cudaError_t rk45(pbe_batch_plan* p, double* N, const pbe_batch_cell_params_t* prm, double t_end,
                 double rtol, double atol, double dt0, int max_attempts, int* steps_out,
                 int* rejects_out, int* attempts_out, cudaStream_t s)
{
    const size_t C = static_cast<size_t>(p->total), nc = static_cast<size_t>(p->n_cells);
    cudaError_t e = cudaSuccess;
    if (!p->rk_k) {
        e = plan_alloc(p, &p->rk_k, 7 * C);
        if (e == cudaSuccess) e = plan_alloc(p, &p->rk_cell, 2 * nc);
        if (e == cudaSuccess) e = plan_alloc(p, &p->rk_int, 3 * nc + 1);
        if (e != cudaSuccess) { p->rk_k = nullptr; return e; }
    }
    Rk45Ctl ctl;
    ctl.t = p->rk_cell;
    ctl.dt = p->rk_cell + nc;
    ctl.status = p->rk_int;
    ctl.steps = p->rk_int + nc;
    ctl.rejects = p->rk_int + 2 * nc;
    ctl.done = p->rk_int + 3 * nc;
    ctl.t_end = t_end;
    ctl.rtol = rtol;
    ctl.atol = atol;
    SelScope scope(p);
    e = sel_cache(p, prm, s);
    if (e != cudaSuccess) return e;
    BatchDev d = p->d;
    d.skip = ctl.status;                   // finished cells: no RHS work
    std::vector<double> init(2 * nc, 0.0);
    for (size_t c = 0; c < nc; ++c) init[nc + c] = std::min(dt0, t_end);
    e = cudaMemcpyAsync(p->rk_cell, init.data(), init.size() * sizeof(double),
                        cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->rk_int, 0, (3 * nc + 1) * sizeof(int), s);
    double* k[7];
    for (int j = 0; j < 7; ++j) k[j] = p->rk_k + static_cast<size_t>(j) * C;
    // first stage of the first step
    if (e == cudaSuccess) e = batch_prep(d, N, prm, kStageRhs, 0.0, 0.0, s);
    if (e == cudaSuccess) e = batch_main(d, N, prm, k[0], false, s);
    StageCombine err{};
    for (int j = 0; j < 7; ++j) { err.k[j] = k[j]; err.a[j] = kDPErr[j]; }
    err.nk = 7;
    err.dt = ctl.dt;
    int attempts = 0, done = 0;
    while (e == cudaSuccess && attempts < max_attempts && done < p->n_cells) {
        const int chunk = std::min(8, max_attempts - attempts);
        for (int a = 0; a < chunk && e == cudaSuccess; ++a) {
            for (int st = 2; st <= 7 && e == cudaSuccess; ++st) {
                StageCombine sc{};
                for (int j = 0; j < st - 1; ++j) { sc.k[j] = k[j]; sc.a[j] = kDP[st - 2][j]; }
                sc.nk = st - 1;
                sc.dt = ctl.dt;
                e = batch_prep_combine(d, N, prm, sc, s);
                if (e == cudaSuccess) e = batch_main(d, d.Y, prm, k[st - 1], false, s);
            }
            if (e == cudaSuccess) e = batch_rk45_control(d, N, d.Y, err, k[0], ctl, s);
        }
        attempts += chunk;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&done, ctl.done, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    if (e == cudaSuccess && steps_out)
        e = cudaMemcpyAsync(steps_out, ctl.steps, nc * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && rejects_out)
        e = cudaMemcpyAsync(rejects_out, ctl.rejects, nc * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (attempts_out) *attempts_out = attempts;
    if (e != cudaSuccess) return e;
    return done == p->n_cells ? cudaSuccess : cudaErrorNotReady;
}

// Work items of the death GEMM: the cells of each grid, largest first, in
// row tiles of 64; each row tile covers the bins below its largest n in
// column tiles of 64.
cudaError_t death_items(pbe_batch_plan* p, cudaStream_t s)
{
    if (p->n_death_items >= 0) return cudaSuccess;
    std::vector<int> gcells;
    std::vector<int4> items;
    for (int g = 0; g < p->n_grids; ++g) {
        std::vector<int> cs;
        for (int c = 0; c < p->n_cells; ++c)
            if (p->cell_grid[c] == g) cs.push_back(c);
        std::stable_sort(cs.begin(), cs.end(),
                         [&](int a, int b) { return p->cell_n[a] > p->cell_n[b]; });
        const int base = static_cast<int>(gcells.size());
        gcells.insert(gcells.end(), cs.begin(), cs.end());
        for (size_t r = 0; r < cs.size(); r += 64) {
            const int rows = static_cast<int>(std::min<size_t>(64, cs.size() - r));
            const int nmax = p->cell_n[cs[r]];
            for (int i0 = 0; i0 < nmax; i0 += 64)
                items.push_back(make_int4(g, base + static_cast<int>(r), rows, i0));
        }
    }
    int4* di = nullptr;
    int* dg = nullptr;
    cudaError_t e = plan_alloc(p, &di, items.size());
    if (e == cudaSuccess) e = plan_alloc(p, &dg, gcells.size());
    if (e == cudaSuccess && !items.empty())
        e = cudaMemcpyAsync(di, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !gcells.empty())
        e = cudaMemcpyAsync(dg, gcells.data(), gcells.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    // k slices so that the GEMM has about 4 CTAs per SM (each CTA's slice
    // still spans >= 256 of the k range)
    int kmax = 0;
    for (int c = 0; c < p->n_cells; ++c) kmax = std::max(kmax, p->cell_n[c]);
    const int want = items.empty() ? 1
        : static_cast<int>((4LL * p->num_sms + static_cast<long long>(items.size()) - 1) /
                           static_cast<long long>(items.size()));
    const int split = std::max(1, std::min({want, 16, (2 * kmax) / 256}));
    double* part = nullptr;
    if (split > 1) {
        e = plan_alloc(p, &part, static_cast<size_t>(split) * static_cast<size_t>(p->total));
        if (e != cudaSuccess) return e;
    }
    // the grids' B matrices (n_g x NC ld_g, ld_g = n_g rounded up to 16),
    // filled once: the GEMM's k loop then only loads its tiles
    const int ncomp = (p->kernel == 5) ? 2 : 1;
    std::vector<long long> hboff(static_cast<size_t>(p->n_grids), 0);
    std::vector<int> used;
    long long btotal = 0;
    for (int g = 0; g < p->n_grids; ++g) {
        bool any = false;
        for (int c = 0; c < p->n_cells && !any; ++c) any = p->cell_grid[c] == g;
        hboff[g] = btotal;
        if (!any) continue;
        used.push_back(g);
        const long long n = p->grid_n[g], ld = (n + 15) / 16 * 16;
        btotal += n * ncomp * ld;
    }
    double* bm = nullptr;
    long long* dbo = nullptr;
    e = plan_alloc(p, &bm, static_cast<size_t>(btotal));
    if (e == cudaSuccess) e = plan_alloc(p, &dbo, hboff.size());
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dbo, hboff.data(), hboff.size() * sizeof(long long),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !used.empty())
        e = batch_death_b(p->d, used.data(), static_cast<int>(used.size()), bm, hboff.data(), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    p->d_death_items = di;
    p->d_gcells = dg;
    p->n_death_items = static_cast<int>(items.size());
    p->death_split = split;
    p->death_part = part;
    p->death_b = bm;
    p->death_boff = dbo;
    return cudaSuccess;
}

} // namespace
} // namespace pbe_gb300

using namespace pbe_gb300;

extern "C" {

int pbe_batch_create(pbe_batch_t* plan, int n_grids, const int* grid_n, const double* grid_x,
                     int n_cells, const int* cell_n, const int* cell_grid, int kernel_type,
                     int selection, int n_quad, const double* t_q, const double* bw_q,
                     int flags, void* stream)
{
    if (!plan) return cudaErrorInvalidValue;
    *plan = nullptr;
    if ((flags & ~(PBE_BATCH_TUNE | PBE_BATCH_RETUNE | PBE_BATCH_BRK_PREP | PBE_BATCH_BRK_TASKS)) ||
        ((flags & PBE_BATCH_BRK_PREP) && (flags & PBE_BATCH_BRK_TASKS)))
        return cudaErrorInvalidValue;
    cudaError_t e = validate(n_grids, grid_n, grid_x, n_cells, cell_n, cell_grid, kernel_type,
                             selection, n_quad, t_q, bw_q);
    if (e != cudaSuccess) return e;
    pbe_batch_plan* p = new (std::nothrow) pbe_batch_plan();
    if (!p) return cudaErrorMemoryAllocation;
    e = create(p, n_grids, grid_n, grid_x, n_cells, cell_n, cell_grid, kernel_type, selection,
               n_quad, t_q, bw_q, flags, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) { destroy(p); return e; }
    *plan = p;
    return cudaSuccess;
}

int pbe_batch_destroy(pbe_batch_t plan)
{
    if (plan) destroy(plan);
    return cudaSuccess;
}

int pbe_batch_offsets(pbe_batch_t plan, long long* offsets)
{
    if (!plan || !offsets) return cudaErrorInvalidValue;
    std::memcpy(offsets, plan->offsets.data(), plan->offsets.size() * sizeof(long long));
    return cudaSuccess;
}

int pbe_batch_rhs(pbe_batch_t plan, const double* N, double* rhs,
                  const pbe_batch_cell_params_t* params, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!N || !rhs || !params) return cudaErrorInvalidDevicePointer;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    SelScope scope(plan);
    e = sel_cache(plan, params, s);
    if (e == cudaSuccess)
        e = batch_prep(plan->d, const_cast<double*>(N), params, kStageRhs, 0.0, 0.0, s);
    if (e == cudaSuccess) e = batch_main(plan->d, N, params, rhs, true, s);
    return e;
}

int pbe_batch_rk4(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params, double dt,
                  int n_steps, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!N || !params) return cudaErrorInvalidDevicePointer;
    if (n_steps < 0 || !std::isfinite(dt)) return cudaErrorInvalidValue;
    if (n_steps == 0) return cudaSuccess;
    return rk4_graph(plan, N, params, dt, n_steps, static_cast<cudaStream_t>(stream));
}

int pbe_batch_rk4_prepare(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params,
                          double dt, int n_steps)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!N || !params) return cudaErrorInvalidDevicePointer;
    if (n_steps <= 0 || !std::isfinite(dt)) return cudaErrorInvalidValue;
    return rk4_capture(plan, N, params, dt, n_steps);
}

int pbe_batch_rk4_percell(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params,
                          double dt, int n_steps, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!N || !params) return cudaErrorInvalidDevicePointer;
    if (n_steps < 0 || !std::isfinite(dt)) return cudaErrorInvalidValue;
    return rk4_percell(plan, N, params, dt, n_steps, static_cast<cudaStream_t>(stream));
}

int pbe_batch_death(pbe_batch_t plan, const double* N, const pbe_batch_cell_params_t* params,
                    double* death, int method, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (plan->kernel < 0 || (method != PBE_DEATH_MOMENTS && method != PBE_DEATH_DMMA))
        return cudaErrorInvalidValue;
    if (!N || !params || !death) return cudaErrorInvalidDevicePointer;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (method == PBE_DEATH_DMMA) {
        e = death_items(plan, s);
        if (e != cudaSuccess) return e;
    }
    return batch_death(plan->d, N, params, death, method, plan->d_death_items,
                       plan->n_death_items, plan->d_gcells, plan->death_part, plan->death_split,
                       plan->total, plan->death_b, plan->death_boff, s);
}

int pbe_batch_rhs_vjp(pbe_batch_t plan, const double* N, const double* lambda, double* gN,
                      double* gparams, const pbe_batch_cell_params_t* params, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!N || !lambda || !gN || !gparams || !params) return cudaErrorInvalidDevicePointer;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    e = vjp_setup(plan, s);
    if (e != cudaSuccess) return e;
    SelScope scope(plan);
    e = sel_cache(plan, params, s);
    if (e != cudaSuccess) return e;
    return batch_vjp(plan->d, plan->vd, N, lambda, gN, gparams, params, s);
}

int pbe_batch_tape_forward(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params,
                           double dt, int n_steps, int checkpoint_every, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!N || !params) return cudaErrorInvalidDevicePointer;
    if (n_steps <= 0 || checkpoint_every <= 0 || !std::isfinite(dt)) return cudaErrorInvalidValue;
    return tape_forward(plan, N, params, dt, n_steps, checkpoint_every,
                        static_cast<cudaStream_t>(stream));
}

int pbe_batch_tape_backward(pbe_batch_t plan, const double* lambda_T, double* gN0,
                            double* gparams, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!plan->t_recorded) return cudaErrorInvalidValue;
    if (!lambda_T || !gN0 || !gparams) return cudaErrorInvalidDevicePointer;
    return tape_backward(plan, lambda_T, gN0, gparams, static_cast<cudaStream_t>(stream));
}

int pbe_batch_rk45(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params,
                   double t_end, double rtol, double atol, double dt0, int max_attempts,
                   int* steps, int* rejects, int* attempts, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!N || !params) return cudaErrorInvalidDevicePointer;
    if (!(t_end > 0.0) || !std::isfinite(t_end) || !(rtol >= 0.0) || !(atol >= 0.0) ||
        !(rtol > 0.0 || atol > 0.0) || !(dt0 > 0.0) || max_attempts <= 0)
        return cudaErrorInvalidValue;
    return rk45(plan, N, params, t_end, rtol, atol, dt0, max_attempts, steps, rejects, attempts,
                static_cast<cudaStream_t>(stream));
}

int pbe_batch_jvp(pbe_batch_t plan, const double* N, const double* v,
                  const pbe_batch_cell_params_t* params, double* out, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!N || !v || !params || !out) return cudaErrorInvalidDevicePointer;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    SelScope scope(plan);
    e = sel_cache(plan, params, s);
    if (e != cudaSuccess) return e;
    return jvp(plan, N, v, params, out, s);
}

int pbe_batch_ros2(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params, double dt,
                   int n_steps, int krylov_dim, double* resid, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!N || !params) return cudaErrorInvalidDevicePointer;
    if (n_steps < 0 || !(dt > 0.0) || !std::isfinite(dt) || krylov_dim < 1 ||
        krylov_dim > kGmresMaxDim)
        return cudaErrorInvalidValue;
    if (n_steps == 0) return cudaSuccess;
    return ros2(plan, N, params, dt, n_steps, krylov_dim, resid, static_cast<cudaStream_t>(stream));
}

int pbe_batch_ros2_adaptive(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params,
                            double t_end, double rtol, double atol, double dt0, int krylov_dim,
                            int max_attempts, int* steps, int* rejects, int* attempts,
                            double* resid, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!N || !params) return cudaErrorInvalidDevicePointer;
    if (!(t_end > 0.0) || !std::isfinite(t_end) || !(rtol >= 0.0) || !(atol >= 0.0) ||
        !(rtol > 0.0 || atol > 0.0) || !(dt0 > 0.0) || max_attempts <= 0 || krylov_dim < 1 ||
        krylov_dim > kGmresMaxDim)
        return cudaErrorInvalidValue;
    return ros2_adaptive(plan, N, params, t_end, rtol, atol, dt0, krylov_dim, max_attempts, steps,
                         rejects, attempts, resid, static_cast<cudaStream_t>(stream));
}

int pbe_batch_set_krylov_tol(pbe_batch_t plan, double tol)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!(tol >= 0.0) || !(tol < 1.0)) return cudaErrorInvalidValue;
    plan->krylov_tol = tol;
    return cudaSuccess;
}

int pbe_batch_set_krylov_restarts(pbe_batch_t plan, int restarts)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (restarts < 0 || restarts > 1000) return cudaErrorInvalidValue;
    plan->krylov_restarts = restarts;
    return cudaSuccess;
}

int pbe_batch_from_soa(pbe_batch_t plan, const double* soa, long long ld, double* N, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!soa || !N) return cudaErrorInvalidDevicePointer;
    if (ld < plan->n_cells) return cudaErrorInvalidValue;
    return batch_soa(plan->d, soa, N, ld, plan->max_n, true, static_cast<cudaStream_t>(stream));
}

int pbe_batch_to_soa(pbe_batch_t plan, const double* N, double* soa, long long ld, void* stream)
{
    cudaError_t e = check_plan(plan);
    if (e != cudaSuccess) return e;
    if (!soa || !N) return cudaErrorInvalidDevicePointer;
    if (ld < plan->n_cells) return cudaErrorInvalidValue;
    return batch_soa(plan->d, N, soa, ld, plan->max_n, false, static_cast<cudaStream_t>(stream));
}

int pbe_batch_schedule(pbe_batch_t plan, int* group_size, int* n_bundles)
{
    if (!plan) return cudaErrorInvalidValue;
    if (group_size) {
        bool present[16] = {false};
        for (int c = 0; c < plan->n_cells; ++c) present[n_class(plan->cell_n[c])] = true;
        for (int c = 0; c < 16; ++c) group_size[c] = present[c] ? plan->group_size[c] : 0;
    }
    if (n_bundles) *n_bundles = plan->d.n_bundles;
    return cudaSuccess;
}

} // extern "C"
