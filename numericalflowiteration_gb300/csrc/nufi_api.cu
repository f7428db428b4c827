// nufi_api.cu — the C ABI of include/nufi_gb300.h: handle lifetime, device
// memory of the coefficient history, and the launch sequence of the hot
// path on one CUDA stream.
//
// Device memory of a handle (all allocated once, in nufi_create):
//   hist     (Nt+1) FP64 slabs, reference layout inside a slab, slab pitch
//            rounded up to 16 bytes; slab n is written by the field solve
//            (nufi_step / nufi_run) or by nufi_upload_phi.
//   tables   (Nt+1) FP32 field tables (split mode only): 1D per cell
//            K(A,B), K C of the spline derivative (store_kick_entry), 2D/3D the FP32 slab.
//   partial  [rows][Ns] FP64 per-block sums of the trace (reduce_rho sums
//            the rows into rho).
//   rho      [Ns] FP64, energy [Nt+1] FP64, err (one error word).
//   solve plan: circulant kernels of the Poisson + collocation diagonal.
//   split tables: per-velocity-node constants and per-cell phases.
#include <chrono>
#include <climits>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "nufi_kernels.cuh"

using namespace nufi_gb300;

namespace {

thread_local std::string g_last_error = "";

}  // namespace

struct nufi_handle {
    nufi_config cfg{};
    nufi_options opt{};
    Problem p{};
    int device = 0;
    cudaStream_t stream = nullptr;
    double *hist = nullptr;
    float *tables = nullptr;
    double *tables64 = nullptr;   // FP64 1D order 4: per-slab derivative tables (trace_fp64_table.cu)
    bool fp64_table = false;      // the FP64 trace runs on tables64
    double *partial = nullptr;
    double *rho = nullptr;
    double *energy = nullptr;
    double *slab_out = nullptr;   // nufi_field_solve scratch
    double *energy_tmp = nullptr; // nufi_field_solve scratch
    unsigned *err = nullptr;
    SplitNode *nodes = nullptr;
    float2 *phase = nullptr;
    double *mpartial = nullptr;  // [4][trace blocks] metrics block sums
    size_t mpartial_n = 0;       // its doubles
    // nufi_set_metrics_grid: the metrics points' grid and its FP64 shape
    bool mgrid_set = false;
    PointGrid mgrid;
    LaunchShape mshape;
    double *metrics = nullptr;   // [4]
    // adjoint (allocated on first nufi_backward)
    AdjointPlan aplan;
    double *mu = nullptr;         // (Nt+1) x P slab adjoints
    double *lambda = nullptr;     // [Ns]
    double *theta_acc = nullptr;  // [4][adjoint blocks]
    double *grad = nullptr;       // [4]
    std::vector<char> slab_set;   // slab n written (step, run, upload_phi)
    // upload_phi's pinned staging slots (one slab each, mapped), the device
    // addresses of the same, and the event after the launch that last read each
    double *stage[2] = {nullptr, nullptr};
    double *stage_dev[2] = {nullptr, nullptr};
    cudaEvent_t stage_done[2] = {nullptr, nullptr};
    // the completion number of the publishing trace that last read each slot
    // (0: another launch read it, wait for its event instead)
    unsigned stage_seq[2] = {0u, 0u};
    int stage_next = 0;
    // 1D split (staged trace): the slab upload_phi staged but has not derived
    // yet (-1: none).  compute_rho(pending_k + 1) derives it inside its trace;
    // every other call that reads the history applies it first (flush_upload).
    long long pending_k = -1;
    int pending_slot = 0;
    // Pinned block of the blocking calls: [0] the device error word (copied
    // on the stream before the one synchronisation of a call), then rho
    // (Ns), the field solve's slab (stride_t) and W, and its rho input (Ns).
    // The *_dev pointers are the block's device addresses: copy_words_kernel
    // moves the small per-step transfers through them.
    double *pin = nullptr;
    unsigned *pin_err = nullptr, *pin_err_dev = nullptr;
    // completion word beside the error word: a kernel that ends a blocking
    // call writes the call's sequence number there after its results
    unsigned *pin_seq = nullptr, *pin_seq_dev = nullptr;
    unsigned seq = 0;      // last sequence number handed out
    unsigned rho_seq = 0;  // the one the published rho carries (0: none, synchronise instead)
    double *pin_rho = nullptr, *pin_slab = nullptr, *pin_rho_in = nullptr;
    double *pin_rho_dev = nullptr, *pin_slab_dev = nullptr, *pin_rho_in_dev = nullptr;
    // value of `launches` right after a compute_rho whose reduction also
    // wrote rho and the error word into the pinned block: while no launch
    // has followed, download_rho only synchronises
    long long rho_pub_at = -1;
    // Speculative field solve: while callers pass nufi_field_solve the rho
    // that the last compute_rho published, compute_rho queues the circulant
    // solve of the device rho behind its trace (results into the pinned
    // block, sequence spec_seq) and field_solve returns them when its input
    // matches that rho bit for bit.  spec_at: `launches` right after that
    // solve (-1: none outstanding).
    bool spec_solve = false;
    unsigned spec_seq = 0;
    long long spec_at = -1;
    std::vector<char> energy_set; // W_n recorded (step, run)
    SolvePlan plan;
    bool solve_ok = false;
    std::string solve_why;
    LaunchShape shape;
    StagedShape staged;
    PersistentRun persist;
    // the staged 1D trace's fixed-point rho (RhoFix): sums [N] and ticket,
    // zero between launches; step_fix_scale == 0: partial rows instead
    unsigned long long *step_fix = nullptr;
    unsigned *step_ticket = nullptr;
    double step_fix_scale = 0, step_fix_limit = 0;
    std::string last_error;
    long long launches = 0;
    std::map<std::pair<long long, long long>, std::pair<cudaGraphExec_t, long long>> graphs;
    std::vector<void *> allocations;
};

namespace {

int create_handle(const nufi_config *cfg, const nufi_options *opt, int device, nufi_handle **out,
                  bool batch_instance);

int fail(nufi_handle *h, int code, const std::string &msg)
{
    if (h) h->last_error = msg;
    else g_last_error = msg;
    return code;
}

int cuda_fail(nufi_handle *h, cudaError_t e, const char *where)
{
    return fail(h, NUFI_ERR_CUDA, std::string(where) + ": " + cudaGetErrorName(e) + ": " + cudaGetErrorString(e));
}

#define NUFI_CUDA(h, call)                                         \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, #call);   \
    } while (0)

template <typename T>
cudaError_t dalloc(nufi_handle *h, T **ptr, size_t count)
{
    void *p = nullptr;
    if (count > SIZE_MAX / sizeof(T)) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T) > 0 ? count * sizeof(T) : 16);
    if (e != cudaSuccess) return e;
    h->allocations.push_back(p);
    *ptr = static_cast<T *>(p);
    return cudaSuccess;
}

// Host-side B-spline basis at x = 0 (collocation stencil N_j(0)).
void stencil(int order, double *Nb)
{
    switch (order) {
#define NUFI_STENCIL(O) \
    case O: bspline_basis<double, O, 0>(0.0, Nb); return;
        NUFI_STENCIL(2) NUFI_STENCIL(3) NUFI_STENCIL(4) NUFI_STENCIL(5) NUFI_STENCIL(6) NUFI_STENCIL(7)
        NUFI_STENCIL(8)
#undef NUFI_STENCIL
    default: break;
    }
}

// k L a multiple of 2 pi, to 2.5e-7 relative (see validate)
bool phase_is_periodic(double k, double L)
{
    const double r = k * L / 6.283185307179586476925286766559;
    return std::fabs(r - std::nearbyint(r)) <= 2.5e-7 * std::max(1.0, std::fabs(r));
}

int validate(const nufi_config *c, std::string &why)
{
    if (!c) { why = "null config"; return NUFI_ERR_INVALID; }
    if (c->dim < 1 || c->dim > 3) { why = "dim must be 1, 2 or 3"; return NUFI_ERR_INVALID; }
    if (c->order < 2 || c->order > kMaxOrder) { why = "order must be in [2, 8]"; return NUFI_ERR_INVALID; }
    if (c->Nt < 0) { why = "Nt must be >= 0"; return NUFI_ERR_INVALID; }
    if (!(c->dt > 0) || !std::isfinite(c->dt)) { why = "dt must be positive and finite"; return NUFI_ERR_INVALID; }
    for (int a = 0; a < c->dim; ++a) {
        if (c->Nx[a] < 1 || c->Nv[a] < 1) { why = "grid sizes must be >= 1"; return NUFI_ERR_INVALID; }
        if (c->Nx[a] > (1 << 20) || c->Nv[a] > kMaxVelocityTable) {
            why = "grid too large (at most 2^20 nodes and 4096 velocity nodes per axis)";
            return NUFI_ERR_RANGE;
        }
        if (!(c->x_max[a] > c->x_min[a]) || !(c->v_max[a] > c->v_min[a])) {
            why = "domain bounds must satisfy min < max";
            return NUFI_ERR_INVALID;
        }
        if (!std::isfinite(c->x_max[a] - c->x_min[a]) || !std::isfinite(c->v_max[a] - c->v_min[a])) {
            why = "domain bounds must be finite";
            return NUFI_ERR_INVALID;
        }
    }
    // Sizes below are products of these counts in 64-bit integers, and the
    // launch shapes hold node and block counts in 32-bit fields: bounded here
    // so that no product wraps (a wrapped allocation size would leave the
    // kernels indexing past their buffers).  A history that merely exceeds
    // the device's memory fails cleanly in cudaMalloc.
    long double ns = 1, nm = 1, slab = 1;
    for (int a = 0; a < c->dim; ++a) {
        ns *= (long double)c->Nx[a];
        nm *= (long double)c->Nv[a];
        slab *= (long double)(c->Nx[a] + c->order - 1);
    }
    if (c->Nt > kMaxSteps) { why = "Nt too large (at most 2^30 time steps)"; return NUFI_ERR_RANGE; }
    if (ns > (long double)INT_MAX || nm > (long double)INT_MAX) {
        why = "grid too large (at most 2^31 - 1 spatial and 2^31 - 1 velocity nodes)";
        return NUFI_ERR_RANGE;
    }
    // 20 bytes per slab value stands for the FP64 history and the FP32
    // tables; with the tables' row padding the real figure is at most 7x
    // that, still far below 2^64
    if (((long double)c->Nt + 1) * (slab + 2) * 20 > (long double)(1ULL << 50)) {
        why = "coefficient history too large (more than 2^50 bytes)";
        return NUFI_ERR_RANGE;
    }
    if (c->precision != NUFI_PREC_FP64 && c->precision != NUFI_PREC_FP32_SPLIT) {
        why = "unknown precision mode";
        return NUFI_ERR_INVALID;
    }
    if (c->f0_kind < NUFI_F0_LANDAU || c->f0_kind > NUFI_F0_BUMP_ON_TAIL) {
        why = "unknown f0 kind";
        return NUFI_ERR_INVALID;
    }
    for (int i = 0; i < 8; ++i)
        if (!std::isfinite(c->f0_params[i])) {
            why = "f0 parameters must be finite";
            return NUFI_ERR_INVALID;
        }
    if (c->f0_kind == NUFI_F0_BUMP_ON_TAIL && !(c->f0_params[3] > 0)) {
        why = "bump-on-tail needs sigma_b > 0";
        return NUFI_ERR_INVALID;
    }
    // 2D: Landau; 3D: Landau and the reference's compiled-in bump-on-tail
    if (c->dim > 1 && c->f0_kind != NUFI_F0_LANDAU && !(c->dim == 3 && c->f0_kind == NUFI_F0_BUMP_ON_TAIL)) {
        why = "f0 kinds other than Landau are 1D only (and bump-on-tail in 3D)";
        return NUFI_ERR_UNSUPPORTED;
    }
    if (c->precision == NUFI_PREC_FP64 && !fp64_order_supported(c->dim, c->order)) {
        why = "FP64 trace not built for this (dim, order)";
        return NUFI_ERR_UNSUPPORTED;
    }
    if (c->precision == NUFI_PREC_FP32_SPLIT && !split_supported(c->dim, c->order, c->f0_kind)) {
        why = "FP32-split trace not built for this (dim, order, f0)";
        return NUFI_ERR_UNSUPPORTED;
    }
    // The FP32-split traces take cos(k x) at the foot from the phase of the
    // cell the foot lands in, i.e. at the foot wrapped into the domain; the
    // reference evaluates f0 at the unwrapped foot (nufi/rho.hpp:59-60).
    // Both agree when k (x_max - x_min) is a multiple of 2 pi on every axis,
    // to 2.5e-7 relative: a domain length rounded to single precision (the
    // reference's <float> configurations: 4 pi in float is 2.8e-8 above 4 pi)
    // passes, and the phase at the foot then moves by at most 2 pi 2.5e-7
    // per wrap of the domain, within the FP32-split form's accuracy.  Other
    // k: the split traces count each chain's wraps per axis and turn the
    // phase by k L_a per wrap (Problem::phase_wrap), for every N_a a power of
    // two (and in 1D up to 256: the staged trace).
    if (c->precision == NUFI_PREC_FP32_SPLIT) {
        bool wraps = false, pow2 = true;
        for (int a = 0; a < c->dim; ++a) {
            wraps = wraps || !phase_is_periodic(c->f0_params[1], c->x_max[a] - c->x_min[a]);
            pow2 = pow2 && (c->Nx[a] & (c->Nx[a] - 1)) == 0;
        }
        if (wraps && (!pow2 || (c->dim == 1 && c->Nx[0] > 256))) {
            why = "FP32-split with k (x_max - x_min) not a multiple of 2 pi: every Nx a power of two (in 1D up to "
                  "256) (f0's phase at the unwrapped foot); the FP64 trace takes any k";
            return NUFI_ERR_UNSUPPORTED;
        }
    }
    return NUFI_OK;
}

Problem make_problem(const nufi_config &c)
{
    Problem p{};
    p.dim = c.dim;
    p.order = c.order;
    p.f0_kind = c.f0_kind;
    p.precision = c.precision;
    p.Ns = 1;
    p.Nm = 1;
    p.stride_t = 1;
    for (int a = 0; a < 3; ++a) {
        const bool in = a < c.dim;
        p.N[a] = in ? int(c.Nx[a]) : 1;
        p.M[a] = in ? int(c.Nv[a]) : 1;
        p.P[a] = in ? int(c.Nx[a] + c.order - 1) : 1;
        // config.hpp:67-69
        p.xmin[a] = in ? c.x_min[a] : 0.0;
        p.L[a] = in ? c.x_max[a] - c.x_min[a] : 1.0;
        p.Linv[a] = 1 / p.L[a];
        p.dx[a] = p.L[a] / p.N[a];
        p.dxinv[a] = 1 / p.dx[a];
        p.vmin[a] = in ? c.v_min[a] : 0.0;
        p.dv[a] = in ? (c.v_max[a] - c.v_min[a]) / p.M[a] : 1.0;
        if (in) {
            p.Ns *= p.N[a];
            p.Nm *= p.M[a];
            p.stride_t *= p.P[a];
        }
    }
    p.Nq = p.Ns * p.Nm;
    p.hist_stride = (p.stride_t + 1) / 2 * 2;
    // 2D/3D FP32 tables: x rows of table_sx floats.  When N[0] < 32 a warp
    // of the split trace spans g = 32 / N[0] x rows, and its gathers take one
    // wavefront only if the rows' N[0] banks are disjoint (with P[0] = N[0]
    // + 3 two 16-node neighbour rows share 3 banks).  The rows a warp holds
    // are row_step = N[1] / g apart (the kernel maps its spatial nodes so),
    // and table_sx is the smallest stride >= P[0] with row_step * table_sx
    // = N[0] (mod 32): 22 instead of 19 for 16^3 (a slab of 31.8 KB), where
    // consecutive rows would need 48 (69.3 KB).  Where no such stride exists
    // the rows are consecutive and table_sx = N[0] (mod 32).
    p.table_sx = p.P[0];
    p.row_step = 0;
    if (c.dim > 1 && p.N[0] < 32) {
        const int g = 32 / p.N[0];
        bool found = false;
        if (32 % p.N[0] == 0 && p.N[1] % g == 0) {
            const int step = p.N[1] / g;
            for (int sx = p.P[0]; sx < p.P[0] + 32 && !found; ++sx)
                if ((1LL * step * sx) % 32 == p.N[0] % 32) {
                    p.table_sx = sx;
                    p.row_step = step;
                    found = true;
                }
        }
        if (!found)
            while (p.table_sx % 32 != p.N[0] % 32) ++p.table_sx;
    }
    p.table_stride = c.dim == 1 ? (3LL * p.N[0] + 3) / 4 * 4 : (1LL * p.table_sx * p.P[1] * p.P[2] + 3) / 4 * 4;
    p.dt = c.dt;
    for (int i = 0; i < 8; ++i) p.f0p[i] = c.f0_params[i];
    p.wv = 1;
    for (int a = 0; a < c.dim; ++a) p.wv *= p.dv[a];
    p.split_plain_kick = 0;  // nufi_options.split_plain_kick, set by the caller
    // 1D split: the phase f0 gains per wrap of the domain (validate admits
    // a non-periodic phase for the staged traces only)
    for (int a = 0; a < 3; ++a) {
        p.phase_wrap[a] = 0.0;
        if (c.precision == NUFI_PREC_FP32_SPLIT && a < c.dim && !phase_is_periodic(c.f0_params[1], p.L[a])) {
            const double two_pi = 6.283185307179586476925286766559, kL = c.f0_params[1] * p.L[a];
            p.phase_wrap[a] = kL - two_pi * std::floor(kL / two_pi);
        }
    }
    return p;
}

// The launch options (nufi_options): NULL = all defaults; any other value
// than the documented ones is refused.
int validate_options(const nufi_options *o, nufi_options &out, std::string &why)
{
    out = nufi_options{};
    if (!o) return NUFI_OK;
    auto flag = [](int32_t v) { return v == 0 || v == 1; };
    if (!flag(o->split_global_loads) || !flag(o->split_plain_kick) || !flag(o->no_persistent) ||
        !flag(o->batch_no_autotune)) {
        why = "options: flags must be 0 or 1";
        return NUFI_ERR_INVALID;
    }
    if (o->split_ctas_per_sm < 0 || o->split_ctas_per_sm > 2 || o->split_threads_per_node < 0 ||
        o->split_threads_per_node > 2) {
        why = "options: split_ctas_per_sm and split_threads_per_node take 0, 1 or 2";
        return NUFI_ERR_INVALID;
    }
    if (o->batch_adjoint_ppt != 0 && o->batch_adjoint_ppt != 1 && o->batch_adjoint_ppt != 2 &&
        o->batch_adjoint_ppt != 4) {
        why = "options: batch_adjoint_ppt takes 0, 1, 2 or 4";
        return NUFI_ERR_INVALID;
    }
    for (int32_t r : o->reserved)
        if (r != 0) {
            why = "options: reserved fields must be 0";
            return NUFI_ERR_INVALID;
        }
    out = *o;
    return NUFI_OK;
}

// Trace tiling: the largest points-per-thread that still gives about four
// resident blocks per SM, then fewer warps per block for small grids.
LaunchShape choose_shape(const Problem &p, int sms)
{
    const long long sblocks = (p.Ns + 31) / 32;
    const int ppts[3] = {4, 2, 1};
    const int warps[3] = {4, 2, 1};
    for (int w : warps)
        for (int ppt : ppts) {
            const long long vb = (p.Nm + (long long)w * ppt - 1) / ((long long)w * ppt);
            if (sblocks * vb >= 4LL * sms) {
                LaunchShape s;
                s.warps = w;
                s.ppt = ppt;
                s.vblocks = int(vb);
                return s;
            }
        }
    LaunchShape s;
    s.warps = 1;
    s.ppt = 1;
    s.vblocks = int(p.Nm);
    return s;
}

// Trace launch shapes for p on a device with `sms` multiprocessors, with no
// CUDA call (nufi_create and nufi_plan).  opt.split_global_loads reads the
// split tables from global memory instead of the shared-memory ring.
void plan_traces(const Problem &p, int sms, const nufi_options &opt, LaunchShape &shape, StagedShape &staged)
{
    shape = choose_shape(p, sms);
    // the FP64 3D cubic trace (trace_fp64_3d_cells_kernel) holds two blocks
    // per SM in 128 registers at up to 2 points per thread; at 4 it spills
    if (p.precision == NUFI_PREC_FP64 && p.dim == 3 && p.order == 4 && shape.ppt > 2) {
        shape.vblocks = int((p.Nm + 2LL * shape.warps - 1) / (2LL * shape.warps));
        shape.ppt = 2;
    }
    staged = StagedShape{};
    const bool no_ring = opt.split_global_loads != 0;
    if (p.precision == NUFI_PREC_FP32_SPLIT && p.dim > 1) {
        staged = staged_shape_nd(p, sms);
        if (no_ring) {
            staged.ring = 0;
            staged.smem = 0;
        }
    } else if (p.precision == NUFI_PREC_FP32_SPLIT && !p.split_plain_kick && !no_ring) {
        staged = staged_shape_1d(p, sms, opt.split_ctas_per_sm == 2 ? 2 : 1, opt.split_threads_per_node == 2 ? 2 : 1);
    }
}

// Shape of the field solve (its node limit and grid), with no CUDA call.
bool solve_geometry(const Problem &p, SolvePlan &pl, std::string &why)
{
    if (p.Ns > kCirculantMaxNodes) {
        // the spectral form: per-axis DFTs, one line per block in shared memory
        for (int a = 0; a < p.dim; ++a)
            if (p.N[a] > kSpectralMaxAxis) {
                why = "device field solve: above 16384 grid nodes every axis must hold at most 4096 nodes";
                return false;
            }
        pl.spectral = true;
        pl.nconv = 2;
        pl.blocks = int((p.Ns + 255) / 256);  // the finishing kernel's blocks (energy parts)
        pl.nodes_per_block = 0;
        pl.smem = 0;
        pl.green_in_smem = false;
        return true;
    }
    pl.nconv = (p.precision == NUFI_PREC_FP32_SPLIT && p.dim == 1) ? 5 : 2;
    // one warp per node; warps (nodes) per block: at most 8, fewer until
    // there are 64 blocks.  Measured on the two-stream grid (256 nodes, the
    // drop-in field solve): 4 nodes per block 18.8 us per call, 1 node
    // 21.1 us, 8 nodes 20.4 us; each block reads rho once (mapped host memory
    // in the drop-in call), so fewer blocks read it fewer times, while more
    // nodes per block serialise more FP64 work on one SM.  The green kernels
    // are read from L2 (batched loads), not staged per block.
    int npb = 8;
    while (npb > 1 && (p.Ns + npb - 1) / npb < 64) npb /= 2;
    pl.nodes_per_block = npb;
    pl.blocks = int((p.Ns + npb - 1) / npb);
    pl.green_in_smem = false;
    pl.smem = size_t(p.Ns) * 8;
    return true;
}

// The whole-run kernel's shape where it applies (1D split with the staged
// trace and the device solve); opt.no_persistent turns it off.
PersistentRun plan_persistent(const Problem &p, const StagedShape &staged, const SolvePlan &plan, bool solve_ok,
                              int sms, const nufi_options &opt)
{
    if (!(solve_ok && staged.ok)) return PersistentRun{};
    if (opt.no_persistent) return PersistentRun{};
    return persistent_shape_1d(p, staged, plan, sms);
}

// The field solve's circulant kernels (see field_solve.cu): for every mode
// k the diagonal D(k) of Poisson (1 / (N |k|^2)) and of Poisson followed by
// the collocation solve (divided by the symbol lambda(k)), then the inverse
// DFT of D, separable per axis, summed in long double.  Even-degree splines
// (orders 3, 5) make lambda vanish at the Nyquist mode, where the
// reference's LSMR from a zero start returns the minimum-norm solution,
// i.e. drops that mode: the same pseudo-inverse here.  In 1D split mode
// three more kernels give K (A, B, C) of the per-cell quadratic directly
// (shifts of c are phase factors of its diagonal).
// The diagonals of the field solve in Fourier space (before the inverse
// DFT of solve_green): [nconv][Ns] complex, long double.
std::vector<std::complex<long double>> solve_diagonals(const Problem &p, int nconv)
{
    const long long Ns = p.Ns;
    using cld = std::complex<long double>;
    const long double two_pi = 6.283185307179586476925286766559005768L;
    double Nb[kMaxOrder] = {0};
    stencil(p.order, Nb);
    // per-axis symbols and |k|^2
    std::vector<std::vector<cld>> lam(p.dim);
    std::vector<std::vector<long double>> ks(p.dim);
    for (int a = 0; a < p.dim; ++a) {
        const int N = p.N[a];
        lam[a].resize(N);
        ks[a].resize(N);
        for (int k = 0; k < N; ++k) {
            cld z(0, 0);
            for (int j = 0; j < p.order; ++j) {
                const long double ang = two_pi * (long double)((long long)j * k % N) / (long double)N;
                z += (long double)Nb[j] * cld(cosl(ang), sinl(ang));
            }
            lam[a][k] = z;
            const long double kf = (2 * k < N) ? (long double)k : (long double)(N - k);
            const long double kk = kf * (two_pi / (long double)p.L[a]);
            ks[a][k] = kk * kk;
        }
    }
    const bool split1d = nconv == 5;  // 1D split: K A, K B, K C follow c and phi
    std::vector<cld> D((size_t)nconv * Ns, cld(0, 0));
    long double lmax = 0;
    for (long long s = 0; s < Ns; ++s) {
        long long r = s;
        cld l(1, 0);
        for (int a = 0; a < p.dim; ++a) {
            l *= lam[a][r % p.N[a]];
            r /= p.N[a];
        }
        lmax = std::max(lmax, std::abs(l));
    }
    const long double K = -(long double)p.dt * p.dt * p.dxinv[0] * p.dxinv[0];
    for (long long s = 1; s < Ns; ++s) {
        long long r = s;
        long double ksq = 0;
        cld l(1, 0);
        int k0 = 0;
        for (int a = 0; a < p.dim; ++a) {
            const int k = int(r % p.N[a]);
            if (a == 0) k0 = k;
            r /= p.N[a];
            ksq += ks[a][k];
            l *= lam[a][k];
        }
        const long double dphi = 1.0L / ((long double)Ns * ksq);
        const cld dc = std::abs(l) <= 1e-12L * lmax ? cld(0, 0) : cld(dphi, 0) / l;
        D[s] = dc;
        D[Ns + s] = cld(dphi, 0);
        if (split1d) {
            const int N = p.N[0];
            auto w = [&](int m) {
                const long double ang = two_pi * (long double)((long long)m * k0 % N) / (long double)N;
                return cld(cosl(ang), sinl(ang));
            };
            D[2 * Ns + s] = (K / 2) * (w(2) - cld(1, 0)) * dc;
            D[3 * Ns + s] = K * (cld(1, 0) - 2.0L * w(1) + w(2)) * dc;
            D[4 * Ns + s] = (K / 2) * (cld(-1, 0) + 3.0L * w(1) - 3.0L * w(2) + w(3)) * dc;
        }
    }
    return D;
}

std::vector<double> solve_green(const Problem &p, int nconv)
{
    using cld = std::complex<long double>;
    const long long Ns = p.Ns;
    const long double two_pi = 6.283185307179586476925286766559005768L;
    std::vector<cld> D = solve_diagonals(p, nconv);
    // inverse DFT (sign +, unnormalised), axis by axis, all kernels
    long long stride = 1;
    for (int a = 0; a < p.dim; ++a) {
        const int N = p.N[a];
        std::vector<cld> tw(N), line(N), out(N);
        for (int k = 0; k < N; ++k) {
            const long double ang = two_pi * (long double)k / (long double)N;
            tw[k] = cld(cosl(ang), sinl(ang));
        }
        for (int c = 0; c < nconv; ++c) {
            cld *base = D.data() + (size_t)c * Ns;
            for (long long l = 0; l < Ns / N; ++l) {
                const long long lo = l % stride, hi = l / stride;
                cld *ptr = base + hi * stride * N + lo;
                for (int k = 0; k < N; ++k) line[k] = ptr[(long long)k * stride];
                for (int i = 0; i < N; ++i) {
                    cld acc(0, 0);
                    for (int k = 0; k < N; ++k) acc += line[k] * tw[(long long)i * k % N];
                    out[i] = acc;
                }
                for (int i = 0; i < N; ++i) ptr[(long long)i * stride] = out[i];
            }
        }
        stride *= N;
    }
    std::vector<double> green((size_t)nconv * Ns);
    for (size_t i = 0; i < green.size(); ++i) green[i] = double(D[i].real());
    return green;
}

int build_solve_plan(nufi_handle *h)
{
    const Problem &p = h->p;
    h->solve_ok = false;
    if (!solve_geometry(p, h->plan, h->solve_why)) return NUFI_OK;
    SolvePlan &pl = h->plan;
    if (pl.spectral) {
        const std::vector<std::complex<long double>> D = solve_diagonals(p, 2);
        std::vector<double2> dg(D.size());
        for (size_t i = 0; i < D.size(); ++i) dg[i] = make_double2(double(D[i].real()), double(D[i].imag()));
        std::vector<double2> tw;
        const long double two_pi = 6.283185307179586476925286766559005768L;
        for (int a = 0; a < p.dim; ++a)
            for (int k = 0; k < p.N[a]; ++k) {
                const long double ang = two_pi * (long double)k / (long double)p.N[a];
                tw.push_back(make_double2(double(cosl(ang)), double(sinl(ang))));
            }
        NUFI_CUDA(h, dalloc(h, &pl.diag, dg.size()));
        NUFI_CUDA(h, dalloc(h, &pl.work, size_t(3) * size_t(p.Ns)));
        NUFI_CUDA(h, dalloc(h, &pl.twiddle, tw.size()));
        NUFI_CUDA(h, dalloc(h, &pl.mean, 1));
        NUFI_CUDA(h, dalloc(h, &pl.energy_partial, size_t(pl.blocks)));
        NUFI_CUDA(h, dalloc(h, &pl.energy_counter, 1));
        NUFI_CUDA(h, cudaMemcpy(pl.diag, dg.data(), dg.size() * sizeof(double2), cudaMemcpyHostToDevice));
        NUFI_CUDA(h, cudaMemcpy(pl.twiddle, tw.data(), tw.size() * sizeof(double2), cudaMemcpyHostToDevice));
        NUFI_CUDA(h, cudaMemset(pl.energy_counter, 0, sizeof(unsigned)));
        NUFI_CUDA(h, field_solve_prepare(pl));
        h->solve_ok = true;
        return NUFI_OK;
    }
    const std::vector<double> green = solve_green(p, h->plan.nconv);
    NUFI_CUDA(h, dalloc(h, &pl.green, green.size()));
    NUFI_CUDA(h, dalloc(h, &pl.energy_partial, size_t(pl.blocks)));
    NUFI_CUDA(h, dalloc(h, &pl.energy_counter, 1));
    NUFI_CUDA(h, cudaMemcpy(pl.green, green.data(), green.size() * sizeof(double), cudaMemcpyHostToDevice));
    NUFI_CUDA(h, cudaMemset(pl.energy_counter, 0, sizeof(unsigned)));
    NUFI_CUDA(h, field_solve_prepare(pl));
    h->solve_ok = true;
    return NUFI_OK;
}

// Per-velocity-node and per-cell constants of the split form (FP64 here).
int build_split_tables(nufi_handle *h)
{
    const Problem &p = h->p;
    std::vector<SplitNode> nodes;
    std::vector<float2> phase;
    const double c0 = 0.39894228040143267793994;
    for (int a = 0; a < p.dim; ++a) {
        for (int j = 0; j < p.M[a]; ++j) {
            SplitNode nd{};
            const double u0 = p.vmin[a] + j * p.dv[a] + p.dv[a] / 2;
            const double w0 = u0 * p.dt / p.dx[a];
            const double S = std::floor(w0);
            const double sig = w0 - S;
            long long S0 = (long long)S % p.N[a];
            if (S0 < 0) S0 += p.N[a];
            nd.u0 = u0;
            nd.u0f = float(u0);
            nd.sig_hi = float(sig);
            nd.sig_lo = float(sig - double(nd.sig_hi));
            nd.S0 = int(S0);
            nd.S0u = int(S);
            const double gm = c0 * std::exp(-u0 * u0 / 2);
            if (p.f0_kind == NUFI_F0_LANDAU) {
                nd.g = 0.39894228040143267793994 * std::exp(-u0 * u0 / 2);
                nd.ga = float(nd.g);
            } else if (p.f0_kind == NUFI_F0_TWO_STREAM) {
                nd.g = 0.39894228040143267793994 * std::exp(-u0 * u0 / 2.) * u0 * u0;
                nd.ga = float(gm);
            } else {
                const double sb = p.f0p[3], z = (u0 - p.f0p[2]) / sb;
                const double g1 = 0.9 * gm, g2 = 0.1 * c0 / sb * std::exp(-z * z / 2);
                nd.g = g1 + g2;
                nd.ga = float(g1);
                nd.gb = float(g2);
            }
            nodes.push_back(nd);
        }
        for (int i = 0; i < p.N[a]; ++i) {
            const double th = p.f0p[1] * (p.xmin[a] + i * p.dx[a]);
            phase.push_back(make_float2(float(std::cos(th)), float(std::sin(th))));
        }
    }
    NUFI_CUDA(h, dalloc(h, &h->nodes, nodes.size()));
    NUFI_CUDA(h, dalloc(h, &h->phase, phase.size()));
    NUFI_CUDA(h, cudaMemcpy(h->nodes, nodes.data(), nodes.size() * sizeof(SplitNode), cudaMemcpyHostToDevice));
    NUFI_CUDA(h, cudaMemcpy(h->phase, phase.data(), phase.size() * sizeof(float2), cudaMemcpyHostToDevice));
    return NUFI_OK;
}

// Turn the device error word `flags` (already read) into a status; a set
// word is cleared on the device.
int device_flags_status(nufi_handle *h, unsigned flags)
{
    if (flags) {
        NUFI_CUDA(h, cudaMemsetAsync(h->err, 0, sizeof(unsigned), h->stream));
        std::string m = "device check failed:";
        if (flags & kErrCellIndex) m += " cell index out of range (non-finite position?)";
        if (flags & kErrKickRange) m += " split-mode kick displacement out of range";
        if (flags & kErrSolveSize) m += " field-solve size";
        if (flags & kErrStageTimeout) m += " shared-memory staging wait timed out";
        if (flags & kErrBarrierTimeout) m += " grid barrier wait timed out";
        if (flags & kErrAdjointRange) m += " adjoint fixed-point sum out of range";
        if (flags & kErrRhoRange) m += " fixed-point rho part out of range";
        *h->pin_err = 0;  // the stream is idle here: nothing writes the block
        h->rho_pub_at = -1;
        return fail(h, NUFI_ERR_DEVICE, m);
    }
    return NUFI_OK;
}

void mark_steps(nufi_handle *h, int64_t n0, int64_t n1, bool energy)
{
    for (int64_t n = n0; n <= n1; ++n) {
        h->slab_set[size_t(n)] = 1;
        if (energy) h->energy_set[size_t(n)] = 1;
    }
}

// Wait for the handle's stream and read its device error word: the word is
// copied on the stream into pinned memory behind the work already queued,
// so one synchronisation covers both.
int sync_and_check(nufi_handle *h)
{
    NUFI_CUDA(h, cudaMemcpyAsync(h->pin_err, h->err, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
    NUFI_CUDA(h, cudaStreamSynchronize(h->stream));
    return device_flags_status(h, *h->pin_err);
}

// As sync_and_check, when the last launch on the stream (launch_copy_words
// with the error word) has already put the word into the pinned block.
int sync_published(nufi_handle *h)
{
    NUFI_CUDA(h, cudaStreamSynchronize(h->stream));
    return device_flags_status(h, *h->pin_err);
}

// The next sequence number for a kernel to write into the completion word
// (never 0, which marks "none").
unsigned next_seq(nufi_handle *h)
{
    if (++h->seq == 0) ++h->seq;
    return h->seq;
}

// Wait for the completion word to reach `seq`: the results and the error
// word the kernel wrote before it are then visible here.  Kernels write
// the word in stream order with increasing numbers, so a later one may
// already have overwritten it (a signed difference >= 0 counts).  About
// 2.4 us sooner than the stream's synchronisation after a short kernel on
// this hardware (the kernel's exit and the stream's completion signal are
// not waited for).  Past 1 ms of polling, the stream's synchronisation
// instead (a long kernel, or one that failed and will never write the word).
int wait_published(nufi_handle *h, unsigned seq)
{
    const auto t0 = std::chrono::steady_clock::now();
    for (unsigned it = 0;; ++it) {
        if (int(__atomic_load_n(h->pin_seq, __ATOMIC_ACQUIRE) - seq) >= 0)
            return device_flags_status(h, *h->pin_err);
        if ((it & 255u) == 255u && std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(1)) break;
    }
    return sync_published(h);
}

// The calling thread's current device set to the handle's for the scope
// of a call (and restored after).
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// Derivation of slab n from a staging slot: one launch reads the slab from
// the mapped pinned slot, writes it into the history and derives its table;
// without a table of that form, a copy and then the derivation.
int derive_staged(nufi_handle *h, int64_t n, int slot)
{
    const Problem &p = h->p;
    double *dst = h->hist + n * p.hist_stride;
    cudaError_t e;
    if (h->tables) {
        e = launch_derive_table(p, h->stage_dev[slot], h->tables + n * p.table_stride, h->stream, dst);
    } else if (h->tables64 && p.dim == 1) {
        e = launch_derive_table64(p, h->stage_dev[slot], h->tables64 + n * fp64_table_stride(p), h->stream, dst);
    } else {
        e = launch_copy_words(h->stage_dev[slot], dst, p.stride_t, nullptr, nullptr, h->stream);
        if (e == cudaSuccess && h->tables64) {
            h->launches += 1;
            e = launch_derive_table64(p, dst, h->tables64 + n * fp64_table_stride(p), h->stream);
        }
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "slab upload launch");
    h->launches += 1;
    NUFI_CUDA(h, cudaEventRecord(h->stage_done[slot], h->stream));
    h->stage_seq[slot] = 0u;
    return NUFI_OK;
}

// Derive a slab upload_phi left pending (before any work that reads the
// history or the tables).
int flush_upload(nufi_handle *h)
{
    if (h->pending_k < 0) return NUFI_OK;
    const long long k = h->pending_k;
    h->pending_k = -1;
    DeviceGuard g(h->device);
    return derive_staged(h, k, h->pending_slot);
}

// The 1D split handles with the staged trace leave the newest upload
// pending: the next compute_rho(n + 1) derives it inside its trace (one
// launch fewer per step of the reference drivers' loop).
bool upload_can_wait(const nufi_handle *h)
{
    return h->p.dim == 1 && h->p.precision == NUFI_PREC_FP32_SPLIT && h->staged.ok && h->step_fix_scale > 0 &&
           h->tables;
}

// Enqueue the trace of step n over [qb, qe) and the reduction into h->rho
// (with `publish`, also into the pinned block with the error word).
int enqueue_trace(nufi_handle *h, long long n, long long qb, long long qe, int mode, bool publish = false)
{
    const Problem &p = h->p;
    cudaError_t e;
    int rows = 0;
    if (!h->staged.ok || p.dim != 1 || p.precision != NUFI_PREC_FP32_SPLIT) {
        const int st = flush_upload(h);
        if (st) return st;
    }
    if (p.precision == NUFI_PREC_FP64 && h->fp64_table && mode == 0)
        e = launch_trace_fp64_table(p, h->shape, h->tables64, h->hist, int(n), qb, qe, h->partial, &rows, h->err,
                                    h->stream);
    else if (p.precision == NUFI_PREC_FP64)
        e = launch_trace_fp64(p, h->shape, h->hist, int(n), qb, qe, mode, h->partial, &rows, h->err, h->stream);
    else if (p.dim > 1)
        e = launch_trace_split_nd(p, h->staged, h->tables, h->nodes, h->phase, int(n), qb, qe, h->partial, &rows,
                                  h->err, h->stream);
    else if (h->staged.ok) {
        PendingSlab pend;
        const int pslot = h->pending_slot;
        if (publish && h->pending_k >= 0 && h->pending_k == n - 1) {  // the trace derives the newest slab itself
            pend.stage = h->stage_dev[pslot];
            pend.k = h->pending_k;
            pend.hist_out = h->hist + pend.k * p.hist_stride;
            pend.table_out = h->tables + pend.k * p.table_stride;
        } else if (h->pending_k >= 0) {
            const int st = flush_upload(h);
            if (st) return st;
        }
        RhoFix fx;
        if (h->step_fix_scale > 0) {
            fx.sum = h->step_fix;
            fx.ticket = h->step_ticket;
            fx.scale = h->step_fix_scale;
            fx.limit = h->step_fix_limit;
            fx.rho = h->rho;
            fx.pub = publish ? h->pin_rho_dev : nullptr;
            fx.err_pub = publish ? h->pin_err_dev : nullptr;
            if (publish) {
                fx.seq_pub = h->pin_seq_dev;
                fx.seq = next_seq(h);
            }
        }
        e = launch_trace_split_staged(p, h->staged, h->tables, h->nodes, h->phase, int(n), qb, qe, h->partial, &rows,
                                      h->err, h->stream, fx, pend);
        if (e == cudaSuccess && pend.k >= 0) {
            h->pending_k = -1;  // derived and stored by the trace; its staging slot is free after it
            NUFI_CUDA(h, cudaEventRecord(h->stage_done[pslot], h->stream));
            h->stage_seq[pslot] = fx.seq;  // every CTA read the slot before the last one wrote seq
        }
    } else
        e = launch_trace_split(p, h->shape, h->tables, h->nodes, h->phase, int(n), qb, qe, h->partial, &rows, h->err,
                               h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "trace launch");
    h->launches += 1;
    if (rows > 0) {  // rows == 0: the trace wrote rho itself (fixed-point sums)
        e = publish ? launch_reduce_rho(p, rows, h->partial, h->rho, h->stream, h->pin_rho_dev, h->err,
                                        h->pin_err_dev)
                    : launch_reduce_rho(p, rows, h->partial, h->rho, h->stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "reduce launch");
        h->launches += 1;
    }
    if (publish) {
        h->rho_seq = rows == 0 ? h->seq : 0u;  // the trace itself wrote rho, the word and seq
        if (h->spec_at >= 0) h->spec_solve = false;  // the last speculative solve went unused
        h->spec_at = -1;
        if (rows == 0 && h->spec_solve && h->solve_ok && !h->plan.spectral) {
            // reads the device rho, writes only the pinned block: rho stays published
            const unsigned s = next_seq(h);
            e = launch_field_solve(p, h->plan, h->rho, h->pin_slab_dev, nullptr, h->pin_slab_dev + p.hist_stride,
                                   h->stream, h->err, h->pin_err_dev, h->pin_seq_dev, s);
            if (e != cudaSuccess) return cuda_fail(h, e, "field solve launch");
            h->launches += 1;
            h->spec_seq = s;
            h->spec_at = h->launches;
        }
        h->rho_pub_at = h->launches;
    }
    return NUFI_OK;
}

int enqueue_step(nufi_handle *h, long long n)
{
    const Problem &p = h->p;
    int st = enqueue_trace(h, n, 0, p.Nq, 0);
    if (st) return st;
    cudaError_t e = launch_field_solve(p, h->plan, h->rho, h->hist + n * p.hist_stride,
                                       h->tables ? h->tables + n * p.table_stride : nullptr, h->energy + n,
                                       h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "field solve launch");
    h->launches += 1;
    if (h->tables64) {
        e = launch_derive_table64(p, h->hist + n * p.hist_stride, h->tables64 + n * fp64_table_stride(p), h->stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "derive table launch");
        h->launches += 1;
    }
    return NUFI_OK;
}


void release(nufi_handle *h)
{
    // a call that returned on the completion word may leave its kernel's
    // last instructions in flight: let the stream drain before freeing
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto &g : h->graphs) cudaGraphExecDestroy(g.second.first);
    h->graphs.clear();
    for (void *p : h->allocations) cudaFree(p);
    h->allocations.clear();
    for (int s = 0; s < 2; ++s) {
        if (h->stage_done[s]) cudaEventSynchronize(h->stage_done[s]);
        if (h->stage[s]) cudaFreeHost(h->stage[s]);
        if (h->stage_done[s]) cudaEventDestroy(h->stage_done[s]);
        h->stage[s] = nullptr;
        h->stage_done[s] = nullptr;
    }
    if (h->pin) cudaFreeHost(h->pin);
    h->pin = nullptr;
    if (h->stream) cudaStreamDestroy(h->stream);
    h->stream = nullptr;
}

}  // namespace

extern "C" {

const char *nufi_last_error(const nufi_handle *h) { return h ? h->last_error.c_str() : g_last_error.c_str(); }

int nufi_create(const nufi_config *cfg, int device, nufi_handle **out)
{
    return nufi_create_ex(cfg, nullptr, device, out);
}

int nufi_create_ex(const nufi_config *cfg, const nufi_options *opt, int device, nufi_handle **out)
{
    return create_handle(cfg, opt, device, out, false);
}

}  // extern "C"

namespace {

// nufi_create_ex; a batch instance (batch_instance) runs on the batch's own
// kernels and gets no FP64 derivative tables.
int create_handle(const nufi_config *cfg, const nufi_options *opt, int device, nufi_handle **out, bool batch_instance)
{
    if (!out) return fail(nullptr, NUFI_ERR_INVALID, "nufi_create: out is null");
    *out = nullptr;
    std::string why;
    int st = validate(cfg, why);
    if (st) return fail(nullptr, st, "nufi_create: " + why);
    nufi_options o{};
    if ((st = validate_options(opt, o, why))) return fail(nullptr, st, "nufi_create: " + why);
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) return fail(nullptr, NUFI_ERR_INVALID, "nufi_create: no such device");
    std::unique_ptr<nufi_handle> h(new nufi_handle);
    h->cfg = *cfg;
    h->opt = o;
    h->device = device;
    h->p = make_problem(*cfg);
    h->p.split_plain_kick = o.split_plain_kick;
    h->fp64_table = !batch_instance && h->p.precision == NUFI_PREC_FP64 && fp64_table_supported(h->p, cfg->Nt);
    DeviceGuard g(device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    plan_traces(h->p, sms > 0 ? sms : 1, h->opt, h->shape, h->staged);
    if (h->p.dim == 1 && phase_wraps(h->p) && !h->staged.ok)
        return fail(nullptr, NUFI_ERR_UNSUPPORTED,
                    "nufi_create: k (x_max - x_min) not a multiple of 2 pi needs the staged FP32-split trace (the "
                    "options chose the global-load form, which takes f0 at the wrapped foot)");
    const Problem &p = h->p;
    // partial-sum rows: the FP64 traces' y blocks (fp64_rows), the global-
    // load split trace's velocity blocks, or the staged traces' CTAs
    const int trace_rows = p.precision == NUFI_PREC_FP64 ? fp64_rows(h->shape) : h->shape.vblocks;
    const size_t partial_rows = size_t(std::max(trace_rows, h->staged.ok ? h->staged.ctas : 0));
    auto bail = [&](int code) {
        g_last_error = h->last_error;
        release(h.get());
        return code;
    };
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(cuda_fail(h.get(), e, "cudaStreamCreate"));
    const size_t nslab = size_t(cfg->Nt + 1);
    if ((e = dalloc(h.get(), &h->hist, nslab * p.hist_stride)) != cudaSuccess ||
        (e = dalloc(h.get(), &h->partial, partial_rows * p.Ns)) != cudaSuccess ||
        (e = dalloc(h.get(), &h->rho, size_t(p.Ns))) != cudaSuccess ||
        (e = dalloc(h.get(), &h->energy, nslab)) != cudaSuccess ||
        (e = dalloc(h.get(), &h->slab_out, size_t(p.hist_stride) + 1)) != cudaSuccess ||
        (e = dalloc(h.get(), &h->mpartial, h->mpartial_n = size_t(4 * ((p.Ns + 31) / 32) * fp64_rows(h->shape)))) !=
            cudaSuccess ||
        (e = dalloc(h.get(), &h->metrics, 4)) != cudaSuccess ||
        (e = dalloc(h.get(), &h->err, 1)) != cudaSuccess)
        return bail(cuda_fail(h.get(), e, "cudaMalloc"));
    h->energy_tmp = h->slab_out + p.hist_stride;  // slab and W leave in one copy
    {
        // regions on 256-byte boundaries: [err][rho Ns][slab hist_stride, W][rho input Ns]
        auto up = [](size_t n) { return (n + 31) & ~size_t(31); };
        const size_t o_rho = 32, o_slab = o_rho + up(size_t(p.Ns)), o_in = o_slab + up(size_t(p.hist_stride) + 1);
        const size_t pin_n = o_in + up(size_t(p.Ns));
        void *pin = nullptr;
        if ((e = cudaMallocHost(&pin, pin_n * sizeof(double))) != cudaSuccess)
            return bail(cuda_fail(h.get(), e, "cudaMallocHost"));
        h->pin = static_cast<double *>(pin);
        h->pin_err = reinterpret_cast<unsigned *>(h->pin);
        *h->pin_err = 0;
        h->pin_seq = reinterpret_cast<unsigned *>(h->pin + 1);
        *h->pin_seq = 0;
        h->pin_rho = h->pin + o_rho;
        h->pin_slab = h->pin + o_slab;
        h->pin_rho_in = h->pin + o_in;
        void *dev = nullptr;
        if ((e = cudaHostGetDevicePointer(&dev, pin, 0)) != cudaSuccess)
            return bail(cuda_fail(h.get(), e, "cudaHostGetDevicePointer"));
        double *pd = static_cast<double *>(dev);
        h->pin_err_dev = reinterpret_cast<unsigned *>(pd);
        h->pin_seq_dev = reinterpret_cast<unsigned *>(pd + 1);
        h->pin_rho_dev = pd + o_rho;
        h->pin_slab_dev = pd + o_slab;
        h->pin_rho_in_dev = pd + o_in;
    }
    if (h->fp64_table && fp64_table_stride(p) > 0) {
        const size_t n64 = nslab * size_t(fp64_table_stride(p));
        if ((e = dalloc(h.get(), &h->tables64, n64)) != cudaSuccess)
            return bail(cuda_fail(h.get(), e, "cudaMalloc"));
        if ((e = cudaMemset(h->tables64, 0, n64 * sizeof(double))) != cudaSuccess)
            return bail(cuda_fail(h.get(), e, "cudaMemset"));
    }
    if (p.precision == NUFI_PREC_FP32_SPLIT) {
        if ((e = dalloc(h.get(), &h->tables, nslab * p.table_stride)) != cudaSuccess)
            return bail(cuda_fail(h.get(), e, "cudaMalloc"));
        if ((st = build_split_tables(h.get()))) return bail(st);
        if ((e = cudaMemset(h->tables, 0, nslab * p.table_stride * sizeof(float))) != cudaSuccess)
            return bail(cuda_fail(h.get(), e, "cudaMemset"));
    }
    if ((e = cudaMemset(h->hist, 0, nslab * p.hist_stride * sizeof(double))) != cudaSuccess ||
        (e = cudaMemset(h->energy, 0, nslab * sizeof(double))) != cudaSuccess ||
        (e = cudaMemset(h->rho, 0, size_t(p.Ns) * sizeof(double))) != cudaSuccess ||
        (e = cudaMemset(h->metrics, 0, 4 * sizeof(double))) != cudaSuccess ||
        (e = cudaMemset(h->err, 0, sizeof(unsigned))) != cudaSuccess)
        return bail(cuda_fail(h.get(), e, "cudaMemset"));
    if ((st = build_solve_plan(h.get()))) return bail(st);
    h->slab_set.assign(nslab, 0);
    h->energy_set.assign(nslab, 0);
    h->aplan = adjoint_plan_1d(p);
    h->persist = plan_persistent(p, h->staged, h->plan, h->solve_ok, sms > 0 ? sms : 1, h->opt);
    if (h->persist.ok && ((e = dalloc(h.get(), &h->persist.sync, 2)) != cudaSuccess ||
                          (e = dalloc(h.get(), &h->persist.epart, nslab * size_t(p.N[0]))) != cudaSuccess ||
                          (e = dalloc(h.get(), &h->persist.rho_fix, 2 * size_t(p.N[0]))) != cudaSuccess))
        return bail(cuda_fail(h.get(), e, "cudaMalloc"));
    if (p.dim == 1 && p.precision == NUFI_PREC_FP32_SPLIT && h->staged.ok &&
        rho_fixed_point(p, h->staged.ctas, h->staged.ppt * h->staged.tpn, h->step_fix_scale, h->step_fix_limit)) {
        if ((e = dalloc(h.get(), &h->step_fix, size_t(p.N[0]))) != cudaSuccess ||
            (e = dalloc(h.get(), &h->step_ticket, 1)) != cudaSuccess ||
            (e = cudaMemset(h->step_fix, 0, size_t(p.N[0]) * sizeof(unsigned long long))) != cudaSuccess ||
            (e = cudaMemset(h->step_ticket, 0, sizeof(unsigned))) != cudaSuccess)
            return bail(cuda_fail(h.get(), e, "cudaMalloc"));
    } else {
        h->step_fix_scale = 0;
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return bail(cuda_fail(h.get(), e, "nufi_create"));
    *out = h.release();
    return NUFI_OK;
}

}  // namespace

extern "C" {

int nufi_destroy(nufi_handle *h)
{
    if (!h) return NUFI_OK;
    {
        DeviceGuard g(h->device);
        if (h->stream) cudaStreamSynchronize(h->stream);
        release(h);
    }
    delete h;
    return NUFI_OK;
}

int nufi_compute_rho(nufi_handle *h, int64_t n, int64_t q_begin, int64_t q_end)
{
    if (!h) return fail(nullptr, NUFI_ERR_INVALID, "null handle");
    if (n < 0 || n > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "Time-step out of range.");
    if (q_begin < 0 || q_end < q_begin || q_end > h->p.Nq)
        return fail(h, NUFI_ERR_RANGE, "quadrature range outside [0, Nq]");
    if (q_begin == q_end) return NUFI_OK;  // as the reference: no launch, rho untouched
    DeviceGuard g(h->device);
    return enqueue_trace(h, n, q_begin, q_end, 0, true);
}

// rho and the error word into the pinned block (one launch), then one
// synchronisation
static int download_rho_impl(nufi_handle *h)
{
    DeviceGuard g(h->device);
    if (h->rho_pub_at != h->launches) {  // something ran after the last compute_rho's reduction
        NUFI_CUDA(h, launch_copy_words(h->rho, h->pin_rho_dev, h->p.Ns, h->err, h->pin_err_dev, h->stream));
        h->launches += 1;
        return sync_published(h);
    }
    return h->rho_seq ? wait_published(h, h->rho_seq) : sync_published(h);
}

int nufi_download_rho(nufi_handle *h, double *rho)
{
    if (!h || !rho) return fail(h, NUFI_ERR_INVALID, "null argument");
    int st = download_rho_impl(h);
    if (st) return st;
    const double *src = h->pin_rho;
    for (long long i = 0; i < h->p.Ns; ++i) rho[i] += src[i];
    return NUFI_OK;
}

int nufi_compute_metrics(nufi_handle *h, int64_t n, int64_t q_begin, int64_t q_end)
{
    if (!h) return fail(nullptr, NUFI_ERR_INVALID, "null handle");
    if (int fst = flush_upload(h)) return fst;  // a pending upload_phi first
    if (n < 0 || n > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "Time-step out of range.");
    const PointGrid grid = h->mgrid_set ? h->mgrid : point_grid_of(h->p);
    if (q_begin < 0 || q_end < q_begin || q_end > grid.Ns * grid.Nm)
        return fail(h, NUFI_ERR_RANGE, "quadrature range outside the metrics grid's [0, Ns Nm]");
    if (q_begin == q_end) return NUFI_OK;  // as the reference: no launch, sums untouched
    DeviceGuard g(h->device);
    const Problem &p = h->p;
    const LaunchShape &shape = h->mgrid_set ? h->mshape : h->shape;
    int rows = 0;
    cudaError_t e = launch_trace_fp64(p, shape, h->hist, int(n), q_begin, q_end, 2, h->mpartial, &rows, h->err,
                                      h->stream, &grid);
    if (e != cudaSuccess) return cuda_fail(h, e, "metrics launch");
    h->launches += 1;
    e = launch_reduce_metrics((grid.Ns + 31) / 32 * (long long)rows, h->mpartial, h->metrics, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "metrics reduce launch");
    h->launches += 1;
    return NUFI_OK;
}

int nufi_set_metrics_grid(nufi_handle *h, const nufi_config *m)
{
    if (!h) return fail(nullptr, NUFI_ERR_INVALID, "null handle");
    if (!m) {
        h->mgrid_set = false;
        return NUFI_OK;
    }
    const Problem &p = h->p;
    if (m->dim != p.dim) return fail(h, NUFI_ERR_INVALID, "nufi_set_metrics_grid: dim must be the handle's");
    PointGrid g = point_grid_of(p);
    g.Ns = 1;
    g.Nm = 1;
    g.w = 1;
    for (int a = 0; a < p.dim; ++a) {
        if (m->Nx[a] < 1 || m->Nv[a] < 1 || !(m->x_max[a] > m->x_min[a]) || !(m->v_max[a] > m->v_min[a]) ||
            !std::isfinite(m->x_max[a] - m->x_min[a]) || !std::isfinite(m->v_max[a] - m->v_min[a]))
            return fail(h, NUFI_ERR_INVALID, "nufi_set_metrics_grid: node counts >= 1 and x_max > x_min, v_max > v_min");
        if (m->Nx[a] > INT32_MAX || m->Nv[a] > INT32_MAX)
            return fail(h, NUFI_ERR_RANGE, "nufi_set_metrics_grid: too many nodes on an axis");
        g.N[a] = int(m->Nx[a]);
        g.M[a] = int(m->Nv[a]);
        g.xmin[a] = m->x_min[a];
        g.dx[a] = (m->x_max[a] - m->x_min[a]) / double(m->Nx[a]);
        g.vmin[a] = m->v_min[a];
        g.dv[a] = (m->v_max[a] - m->v_min[a]) / double(m->Nv[a]);
        g.Ns *= m->Nx[a];
        g.Nm *= m->Nv[a];
        if (g.Ns > INT32_MAX || g.Nm > INT32_MAX)
            return fail(h, NUFI_ERR_RANGE, "nufi_set_metrics_grid: at most 2^31 - 1 spatial and velocity points");
    }
    for (int a = 0; a < p.dim; ++a) g.w *= g.dv[a];  // as Problem::wv, then dx below 3D (point_grid_of)
    if (p.dim < 3)
        for (int a = 0; a < p.dim; ++a) g.w *= g.dx[a];
    DeviceGuard dg(h->device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    Problem q = p;
    q.Ns = g.Ns;
    q.Nm = g.Nm;
    const LaunchShape shape = choose_shape(q, sms > 0 ? sms : 1);
    const size_t need = size_t(4) * size_t((g.Ns + 31) / 32) * size_t(fp64_rows(shape));
    if (need > h->mpartial_n) {
        // the old buffer may still be read by queued work: it stays allocated
        // until the handle is destroyed
        NUFI_CUDA(h, dalloc(h, &h->mpartial, need));
        h->mpartial_n = need;
    }
    h->mgrid = g;
    h->mshape = shape;
    h->mgrid_set = true;
    return NUFI_OK;
}

int nufi_download_metrics(nufi_handle *h, double *metrics4)
{
    if (!h || !metrics4) return fail(h, NUFI_ERR_INVALID, "null argument");
    DeviceGuard g(h->device);
    double tmp[4];
    NUFI_CUDA(h, cudaMemcpyAsync(tmp, h->metrics, sizeof(tmp), cudaMemcpyDeviceToHost, h->stream));
    int st = sync_and_check(h);
    if (st) return st;
    for (int k = 0; k < 4; ++k) metrics4[k] += tmp[k];
    return NUFI_OK;
}

int nufi_download_rho_f32(nufi_handle *h, float *rho)
{
    if (!h || !rho) return fail(h, NUFI_ERR_INVALID, "null argument");
    int st = download_rho_impl(h);
    if (st) return st;
    const double *src = h->pin_rho;
    for (long long i = 0; i < h->p.Ns; ++i) rho[i] += float(src[i]);
    return NUFI_OK;
}

// The slab goes through a pinned staging slot (two, in turn), so the call
// returns as soon as the caller's buffer has been read (as the reference's
// blocking copy), and the transfer and table derivation stay ordered on the
// stream before the next trace.  A slot is reused after the launch that last
// read it has completed (its event).
//
static int upload_slab(nufi_handle *h, int64_t n, const double *slab)
{
    const Problem &p = h->p;
    DeviceGuard g(h->device);
    int st = flush_upload(h);  // an older pending slab is derived now (from the other slot)
    if (st) return st;
    const size_t bytes = size_t(p.stride_t) * sizeof(double);
    const int slot = h->stage_next;
    h->stage_next ^= 1;
    if (!h->stage[slot]) {
        NUFI_CUDA(h, cudaMallocHost(&h->stage[slot], bytes));
        void *dev = nullptr;
        NUFI_CUDA(h, cudaHostGetDevicePointer(&dev, h->stage[slot], 0));
        h->stage_dev[slot] = static_cast<double *>(dev);
        NUFI_CUDA(h, cudaEventCreateWithFlags(&h->stage_done[slot], cudaEventDisableTiming));
    } else if (!h->stage_seq[slot] || int(__atomic_load_n(h->pin_seq, __ATOMIC_ACQUIRE) - h->stage_seq[slot]) < 0) {
        // the slot's reader has not been seen to finish through the
        // completion word (a read of the pinned word; the event's
        // synchronisation costs ~2 us even when it has completed)
        NUFI_CUDA(h, cudaEventSynchronize(h->stage_done[slot]));
    }
    std::memcpy(h->stage[slot], slab, bytes);
    h->slab_set[size_t(n)] = 1;
    if (upload_can_wait(h)) {
        h->pending_k = n;
        h->pending_slot = slot;
        return NUFI_OK;
    }
    return derive_staged(h, n, slot);
}

int nufi_upload_phi(nufi_handle *h, int64_t n, const double *coeffs_base)
{
    if (!h || !coeffs_base) return fail(h, NUFI_ERR_INVALID, "null argument");
    if (n < 0 || n > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "Time-step out of range.");
    return upload_slab(h, n, coeffs_base + n * h->p.stride_t);
}

int nufi_upload_phi_f32(nufi_handle *h, int64_t n, const float *coeffs_base)
{
    if (!h || !coeffs_base) return fail(h, NUFI_ERR_INVALID, "null argument");
    if (n < 0 || n > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "Time-step out of range.");
    std::vector<double> tmp(size_t(h->p.stride_t));
    const float *src = coeffs_base + n * h->p.stride_t;
    for (size_t i = 0; i < tmp.size(); ++i) tmp[i] = double(src[i]);
    return upload_slab(h, n, tmp.data());
}

int nufi_step(nufi_handle *h, int64_t n, double *energy)
{
    if (!h) return fail(nullptr, NUFI_ERR_INVALID, "null handle");
    if (int fst = flush_upload(h)) return fst;  // a pending upload_phi first
    if (n < 0 || n > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "Time-step out of range.");
    if (!h->solve_ok) return fail(h, NUFI_ERR_UNSUPPORTED, h->solve_why);
    DeviceGuard g(h->device);
    int st = enqueue_step(h, n);
    if (st) return st;
    mark_steps(h, n, n, true);
    if (energy) {
        NUFI_CUDA(h, cudaMemcpyAsync(energy, h->energy + n, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        return sync_and_check(h);
    }
    return NUFI_OK;
}

int nufi_run(nufi_handle *h, int64_t n0, int64_t n1, double *energy_hist)
{
    if (!h) return fail(nullptr, NUFI_ERR_INVALID, "null handle");
    if (int fst = flush_upload(h)) return fst;  // a pending upload_phi first
    if (n0 < 0 || n1 < n0 || n1 > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "step range outside [0, Nt]");
    if (!h->solve_ok) return fail(h, NUFI_ERR_UNSUPPORTED, h->solve_why);
    DeviceGuard g(h->device);
    if (h->persist.ok) {
        // one cooperative launch for all steps (run_split_1d.cu)
        const Problem &p = h->p;
        cudaError_t e = launch_run_split_1d(p, h->persist, h->plan, h->tables, h->hist, h->nodes, h->phase, h->rho,
                                            h->energy, int(n0), int(n1), h->err, h->stream);
        if (e == cudaSuccess) {
            h->launches += 1;
            mark_steps(h, n0, n1, true);
            if (energy_hist) {
                NUFI_CUDA(h, cudaMemcpyAsync(energy_hist, h->energy + n0, size_t(n1 - n0 + 1) * sizeof(double),
                                             cudaMemcpyDeviceToHost, h->stream));
                return sync_and_check(h);
            }
            return NUFI_OK;
        }
        if (e != cudaErrorCooperativeLaunchTooLarge && e != cudaErrorNotSupported)
            return cuda_fail(h, e, "persistent run launch");
        cudaGetLastError();
        h->persist.ok = false;  // fall back to the graph of per-step launches
    }
    const auto key = std::make_pair((long long)n0, (long long)n1);
    auto it = h->graphs.find(key);
    if (it == h->graphs.end()) {
        cudaGraph_t graph = nullptr;
        const long long before = h->launches;
        NUFI_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        int st = NUFI_OK;
        for (int64_t n = n0; n <= n1 && st == NUFI_OK; ++n) st = enqueue_step(h, n);
        cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
        const long long per_launch = h->launches - before;
        h->launches = before;
        if (st) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
        cudaGraphExec_t exec = nullptr;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
        it = h->graphs.emplace(key, std::make_pair(exec, per_launch)).first;
    }
    NUFI_CUDA(h, cudaGraphLaunch(it->second.first, h->stream));
    h->launches += it->second.second;
    mark_steps(h, n0, n1, true);
    if (energy_hist) {
        NUFI_CUDA(h, cudaMemcpyAsync(energy_hist, h->energy + n0, size_t(n1 - n0 + 1) * sizeof(double),
                                     cudaMemcpyDeviceToHost, h->stream));
        return sync_and_check(h);
    }
    return NUFI_OK;
}

int nufi_download_history(nufi_handle *h, int64_t n0, int64_t n1, double *coeffs_base)
{
    if (!h || !coeffs_base) return fail(h, NUFI_ERR_INVALID, "null argument");
    if (int fst = flush_upload(h)) return fst;  // a pending upload_phi first
    if (n0 < 0 || n1 < n0 || n1 > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "step range outside [0, Nt]");
    const Problem &p = h->p;
    DeviceGuard g(h->device);
    NUFI_CUDA(h, cudaMemcpy2DAsync(coeffs_base + n0 * p.stride_t, size_t(p.stride_t) * sizeof(double),
                                   h->hist + n0 * p.hist_stride, size_t(p.hist_stride) * sizeof(double),
                                   size_t(p.stride_t) * sizeof(double), size_t(n1 - n0 + 1),
                                   cudaMemcpyDeviceToHost, h->stream));
    return sync_and_check(h);
}

int nufi_download_energy(nufi_handle *h, int64_t n0, int64_t n1, double *energy)
{
    if (!h || !energy) return fail(h, NUFI_ERR_INVALID, "null argument");
    if (n0 < 0 || n1 < n0 || n1 > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "step range outside [0, Nt]");
    DeviceGuard g(h->device);
    NUFI_CUDA(h, cudaMemcpyAsync(energy, h->energy + n0, size_t(n1 - n0 + 1) * sizeof(double),
                                 cudaMemcpyDeviceToHost, h->stream));
    return sync_and_check(h);
}

int nufi_field_solve(nufi_handle *h, const double *rho, double *slab_out, double *energy)
{
    if (!h || !rho || !slab_out) return fail(h, NUFI_ERR_INVALID, "null argument");
    if (!h->solve_ok) return fail(h, NUFI_ERR_UNSUPPORTED, h->solve_why);
    const Problem &p = h->p;
    DeviceGuard g(h->device);
    const size_t rho_bytes = size_t(p.Ns) * sizeof(double);
    if (h->spec_at >= 0) {
        const bool current = h->spec_at == h->launches;  // nothing launched since the speculative solve
        h->spec_at = -1;
        if (current) {
            int st = wait_published(h, h->spec_seq);  // the trace's rho and the solve's results
            if (st) return st;
            if (std::memcmp(rho, h->pin_rho, rho_bytes) == 0) {  // the same input: the same results
                std::memcpy(slab_out, h->pin_slab, size_t(p.stride_t) * sizeof(double));
                if (energy) *energy = h->pin_slab[p.hist_stride];
                return NUFI_OK;
            }
        }
        h->spec_solve = false;
    }
    // Every call leaves with its copies complete (synchronised, also on
    // failure), so the pinned input is free to overwrite here.
    // The solve reads rho straight from the mapped pinned block; the
    // circulant form also writes the slab, W and the error word there (one
    // launch), the spectral form into device memory and a copy follows.
    std::memcpy(h->pin_rho_in, rho, size_t(p.Ns) * sizeof(double));
    cudaError_t e;
    const char *what = "field solve launch";
    unsigned seq = 0;
    if (!h->plan.spectral) {
        seq = next_seq(h);
        e = launch_field_solve(p, h->plan, h->pin_rho_in_dev, h->pin_slab_dev, nullptr, h->pin_slab_dev + p.hist_stride,
                               h->stream, h->err, h->pin_err_dev, h->pin_seq_dev, seq);
        if (e == cudaSuccess) h->launches += 1;
    } else {
        e = launch_field_solve(p, h->plan, h->pin_rho_in_dev, h->slab_out, nullptr, h->energy_tmp, h->stream);
        if (e == cudaSuccess) {  // slab and W (adjacent on the device) and the error word in one launch
            h->launches += 1;
            e = launch_copy_words(h->slab_out, h->pin_slab_dev, p.hist_stride + 1, h->err, h->pin_err_dev,
                                  h->stream);
            what = "slab copy";
            if (e == cudaSuccess) h->launches += 1;
        }
    }
    if (e != cudaSuccess) {
        cudaStreamSynchronize(h->stream);
        return cuda_fail(h, e, what);
    }
    int st = seq ? wait_published(h, seq) : sync_published(h);
    if (st) return st;
    std::memcpy(slab_out, h->pin_slab, size_t(p.stride_t) * sizeof(double));
    if (energy) *energy = h->pin_slab[p.hist_stride];
    // the input was the rho the last compute_rho published (its trace is
    // complete here): speculate from the next compute_rho on
    if (seq && h->rho_seq && h->rho_pub_at >= 0 && std::memcmp(h->pin_rho_in, h->pin_rho, rho_bytes) == 0)
        h->spec_solve = true;
    return NUFI_OK;
}

int nufi_synchronize(nufi_handle *h)
{
    if (!h) return fail(nullptr, NUFI_ERR_INVALID, "null handle");
    if (int fst = flush_upload(h)) return fst;  // a pending upload_phi first
    DeviceGuard g(h->device);
    return sync_and_check(h);
}

int nufi_sizes(const nufi_handle *h, int64_t *stride_t, int64_t *n_spatial, int64_t *n_points)
{
    if (!h) return fail(nullptr, NUFI_ERR_INVALID, "null handle");
    if (stride_t) *stride_t = h->p.stride_t;
    if (n_spatial) *n_spatial = h->p.Ns;
    if (n_points) *n_points = h->p.Nq;
    return NUFI_OK;
}

int nufi_stream(const nufi_handle *h, void **stream)
{
    if (!h || !stream) return fail(nullptr, NUFI_ERR_INVALID, "null argument");
    // the caller's own work on the stream may read the history: a pending
    // upload_phi is launched first (the handle's state, not its identity)
    if (int fst = flush_upload(const_cast<nufi_handle *>(h))) return fst;
    *stream = static_cast<void *>(h->stream);
    return NUFI_OK;
}

int nufi_launch_count(const nufi_handle *h, int64_t *count)
{
    if (!h || !count) return fail(nullptr, NUFI_ERR_INVALID, "null argument");
    *count = h->launches;
    return NUFI_OK;
}

int nufi_objective(nufi_handle *h, int64_t n1, double *J)
{
    if (!h || !J) return fail(h, NUFI_ERR_INVALID, "null argument");
    if (int fst = flush_upload(h)) return fst;  // a pending upload_phi first
    if (n1 < 0 || n1 > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "step outside [0, Nt]");
    for (int64_t n = 0; n <= n1; ++n)
        if (!h->energy_set[size_t(n)])
            return fail(h, NUFI_ERR_RANGE, "objective: W_n of steps 0..n1 not computed (run the forward first)");
    DeviceGuard g(h->device);
    std::vector<double> w(size_t(n1 + 1));
    NUFI_CUDA(h, cudaMemcpyAsync(w.data(), h->energy, w.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    int st = sync_and_check(h);
    if (st) return st;
    double s = 0;
    for (double v : w) s += v;
    *J = 2.0 * h->cfg.dt * s;
    return NUFI_OK;
}

int nufi_forward(nufi_handle *h, int64_t n1, double *J)
{
    int st = nufi_run(h, 0, n1, nullptr);
    if (st) return st;
    return J ? nufi_objective(h, n1, J) : NUFI_OK;
}

int nufi_backward(nufi_handle *h, int64_t n1, double *grad)
{
    if (!h || !grad) return fail(h, NUFI_ERR_INVALID, "null argument");
    if (int fst = flush_upload(h)) return fst;  // a pending upload_phi first
    if (n1 < 0 || n1 > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "step outside [0, Nt]");
    if (!h->aplan.ok)
        return fail(h, NUFI_ERR_UNSUPPORTED, "backward: built for 1D, orders 4 and 6 (odd-degree splines)");
    if (!h->solve_ok) return fail(h, NUFI_ERR_UNSUPPORTED, h->solve_why);
    if (h->plan.spectral)
        return fail(h, NUFI_ERR_UNSUPPORTED, "backward: grids of at most 16384 nodes (the circulant field solve)");
    for (int64_t n = 0; n <= n1; ++n)
        if (!h->slab_set[size_t(n)])
            return fail(h, NUFI_ERR_RANGE, "backward: slabs 0..n1 not present (run the forward first)");
    DeviceGuard g(h->device);
    const Problem &p = h->p;
    const AdjointPlan &ap = h->aplan;
    const size_t blocks = size_t(ap.grid_x) * ap.grid_y;
    const size_t mu_n = size_t(h->cfg.Nt + 1) * p.P[0];
    if (!h->mu) {
        cudaError_t e;
        if ((e = dalloc(h, &h->mu, mu_n)) != cudaSuccess || (e = dalloc(h, &h->lambda, size_t(p.Ns))) != cudaSuccess ||
            (e = dalloc(h, &h->theta_acc, 4 * blocks)) != cudaSuccess || (e = dalloc(h, &h->grad, 4)) != cudaSuccess)
            return cuda_fail(h, e, "cudaMalloc");
    }
    NUFI_CUDA(h, cudaMemsetAsync(h->mu, 0, mu_n * sizeof(double), h->stream));
    NUFI_CUDA(h, cudaMemsetAsync(h->theta_acc, 0, 4 * blocks * sizeof(double), h->stream));
    cudaError_t e = launch_adjoint_1d(p, ap, h->hist, h->plan.green, h->mu, h->lambda, h->theta_acc, int(n1), h->err,
                                      h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "adjoint launch");
    h->launches += 2 * (n1 + 1);
    e = launch_reduce_metrics((long long)blocks, h->theta_acc, h->grad, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "adjoint reduce launch");
    h->launches += 1;
    NUFI_CUDA(h, cudaMemcpyAsync(grad, h->grad, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    return sync_and_check(h);
}

int nufi_eval_points(nufi_handle *h, int64_t n, int mode, int64_t npts, const double *pts, double *f_out,
                     double *feet)
{
    if (!h || (npts > 0 && !pts)) return fail(h, NUFI_ERR_INVALID, "null argument");
    if (int fst = flush_upload(h)) return fst;  // a pending upload_phi first
    if (n < 0 || n > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "Time-step out of range.");
    if (mode < NUFI_EVAL_FTILDA || mode > NUFI_EVAL_PHASE_FLOW || (mode == NUFI_EVAL_PHASE_FLOW && h->p.dim != 1))
        return fail(h, NUFI_ERR_INVALID, "eval_points: mode (phase flow is 1D, as the reference's)");
    if (npts < 0) return fail(h, NUFI_ERR_INVALID, "eval_points: npts < 0");
    if (npts == 0) return NUFI_OK;
    // buffer bytes and the launch's block count stay far from wrapping
    if (npts > kMaxEvalPoints) return fail(h, NUFI_ERR_RANGE, "eval_points: more than 2^36 points in one call");
    DeviceGuard g(h->device);
    const int D = h->p.dim;
    const size_t pbytes = size_t(npts) * 2 * D * sizeof(double);
    double *dp = nullptr, *df = nullptr, *dfeet = nullptr;
    auto cleanup = [&] {
        cudaFree(dp);
        cudaFree(df);
        cudaFree(dfeet);
    };
    cudaError_t e;
    if ((e = cudaMalloc(&dp, pbytes)) != cudaSuccess ||
        (f_out && mode != NUFI_EVAL_PHASE_FLOW && (e = cudaMalloc(&df, size_t(npts) * sizeof(double))) != cudaSuccess) ||
        (feet && (e = cudaMalloc(&dfeet, pbytes)) != cudaSuccess)) {
        cleanup();
        return cuda_fail(h, e, "cudaMalloc");
    }
    e = cudaMemcpyAsync(dp, pts, pbytes, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = launch_eval_points(h->p, h->hist, int(n), mode, (long long)npts, dp, df, dfeet, h->err, h->stream);
    if (e == cudaSuccess && df)
        e = cudaMemcpyAsync(f_out, df, size_t(npts) * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && dfeet) e = cudaMemcpyAsync(feet, dfeet, pbytes, cudaMemcpyDeviceToHost, h->stream);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(h->stream);
        cleanup();
        return cuda_fail(h, e, "eval_points");
    }
    h->launches += 1;
    const int st = sync_and_check(h);
    cleanup();
    return st;
}

// Coefficient history as text in the reference's layout
// (bin/test_nufi_cpu_3d_isolated.cpp:64-72, 190-211): seven header lines
// "Nt = ", "dt = ", "Nx = ", "Ny = ", "Nz = ", "order = " and a blank one,
// then every coefficient of slabs 0..Nt, one per line, slab after slab.
// As the reference, the header's Nt is the configuration's Nt and dt is
// printed as std::to_string prints it (six decimals); the reference's
// reader takes Nt + 1 slabs whatever the header says, so slabs after n1
// (not computed yet) are written as zeros.  Values carry 17 significant
// digits, so FP64 values read back exactly.
int nufi_save_history(nufi_handle *h, int64_t n1, const char *path)
{
    if (!h || !path) return fail(h, NUFI_ERR_INVALID, "null argument");
    if (int fst = flush_upload(h)) return fst;  // a pending upload_phi first
    if (n1 < 0 || n1 > h->cfg.Nt) return fail(h, NUFI_ERR_RANGE, "step outside [0, Nt]");
    const Problem &p = h->p;
    std::vector<double> all(size_t(n1 + 1) * p.stride_t);
    int st = nufi_download_history(h, 0, n1, all.data());
    if (st) return st;
    FILE *f = std::fopen(path, "w");
    if (!f) return fail(h, NUFI_ERR_INVALID, std::string("save_history: cannot open ") + path);
    std::fprintf(f, "Nt = %lld\ndt = %f\nNx = %d\nNy = %d\nNz = %d\norder = %d\n\n", (long long)h->cfg.Nt, p.dt,
                 p.N[0], p.dim > 1 ? p.N[1] : 1, p.dim > 2 ? p.N[2] : 1, p.order);
    for (double v : all) std::fprintf(f, "%.17g\n", v);
    for (long long i = (long long)(n1 + 1) * p.stride_t; i < (long long)(h->cfg.Nt + 1) * p.stride_t; ++i)
        std::fputs("0\n", f);
    const bool ok = std::fclose(f) == 0;
    return ok ? NUFI_OK : fail(h, NUFI_ERR_INVALID, "save_history: write failed");
}

// Reads such a file (or one without the header, as bin/test_nufi_gpu_1d.cpp
// writes) and uploads its slabs 0..n-1; *n_slabs = n, where trailing
// all-zero slabs (the steps a partial save had not computed) are not
// counted, so a resumed run starts at step n.  A header that disagrees
// with the handle's grid or order is NUFI_ERR_INVALID.
int nufi_load_history(nufi_handle *h, const char *path, int64_t *n_slabs)
{
    if (!h || !path) return fail(h, NUFI_ERR_INVALID, "null argument");
    if (int fst = flush_upload(h)) return fst;  // a pending upload_phi first
    const Problem &p = h->p;
    FILE *f = std::fopen(path, "r");
    if (!f) return fail(h, NUFI_ERR_INVALID, std::string("load_history: cannot open ") + path);
    std::vector<double> vals;
    long long hdr[4] = {-1, -1, -1, -1};  // Nx Ny Nz order
    // whole lines of any length (the reference reads whitespace-separated
    // values with >>, so a line may hold many of them)
    std::string line;
    char chunk[512];
    auto next_line = [&]() -> bool {
        line.clear();
        while (std::fgets(chunk, sizeof(chunk), f)) {
            line += chunk;
            if (line.back() == '\n') return true;
        }
        return !line.empty();
    };
    while (next_line()) {
        char key[32];
        double v;
        if (std::sscanf(line.c_str(), " %31[A-Za-z] = %lf", key, &v) == 2) {
            const std::string k = key;
            if (k == "Nx") hdr[0] = (long long)v;
            else if (k == "Ny") hdr[1] = (long long)v;
            else if (k == "Nz") hdr[2] = (long long)v;
            else if (k == "order") hdr[3] = (long long)v;
            continue;
        }
        const char *s = line.c_str();
        char *end = nullptr;
        for (;;) {
            const double x = std::strtod(s, &end);
            if (end == s) break;
            vals.push_back(x);
            s = end;
        }
    }
    std::fclose(f);
    const long long want[4] = {p.N[0], p.dim > 1 ? p.N[1] : 1, p.dim > 2 ? p.N[2] : 1, p.order};
    for (int i = 0; i < 4; ++i)
        if (hdr[i] >= 0 && hdr[i] != want[i])
            return fail(h, NUFI_ERR_INVALID, "load_history: header does not match the handle's grid or order");
    long long ns = (long long)(vals.size() / size_t(p.stride_t));
    if (ns < 1 || ns > h->cfg.Nt + 1)
        return fail(h, NUFI_ERR_RANGE, "load_history: no whole slab, or more than Nt + 1 slabs");
    while (ns > 1) {  // drop trailing all-zero slabs
        const double *sl = vals.data() + (ns - 1) * p.stride_t;
        if (!std::all_of(sl, sl + p.stride_t, [](double v) { return v == 0.0; })) break;
        --ns;
    }
    for (long long n = 0; n < ns; ++n) {
        const int st = upload_slab(h, n, vals.data() + n * p.stride_t);
        if (st) return st;
    }
    if (n_slabs) *n_slabs = ns;
    return NUFI_OK;
}

}  // extern "C"

namespace {

// The launch plan of a handle as JSON (nufi_describe); with `layout`, also
// the device layout and the adjoint's grid (nufi_plan).
std::string plan_json(const nufi_handle *h, bool layout)
{
    const Problem &p = h->p;
    char tmp[1024];
    const char *fp64_trace = !h->fp64_table ? "trace_fp64_kernel"
                             : p.dim == 1   ? "trace_fp64_1d_table_kernel"
                             : p.dim == 2   ? "trace_fp64_2d_table_kernel"
                                            : "trace_fp64_3d_cells_kernel";
    const char *trace = p.precision == NUFI_PREC_FP64 ? fp64_trace
                        : p.dim > 1                   ? "trace_split_nd_kernel"
                        : h->staged.ok                ? "trace_split_1d_staged_kernel"
                                                      : "trace_split_1d_kernel";
    int k = std::snprintf(
        tmp, sizeof(tmp),
        "{\"trace\": \"%s\", \"fp64_shape\": {\"warps\": %d, \"ppt\": %d, \"vblocks\": %d}, "
        "\"staged\": {\"ok\": %d, \"ctas\": %d, \"threads\": %d, \"ppt\": %d, \"slabs_per_chunk\": %d, "
        "\"ring\": %d, \"smem\": %zu}, \"run\": \"%s\", \"persistent\": {\"ok\": %d, \"ctas\": %d, "
        "\"threads\": %d, \"ppt\": %d, \"smem\": %zu}, \"solve\": {\"ok\": %d, \"kernel\": "
        "\"%s<%d>\", \"blocks\": %d, \"nodes_per_block\": %d}}",
        trace, h->shape.warps, h->shape.ppt, h->shape.vblocks, int(h->staged.ok), h->staged.ctas,
        h->staged.threads, h->staged.ppt, h->staged.slabs_per_chunk, h->staged.ring, h->staged.smem,
        h->persist.ok ? "run_split_1d_kernel" : "graph of per-step launches", int(h->persist.ok), h->persist.ctas,
        h->persist.threads, h->persist.ppt, h->persist.smem, int(h->solve_ok),
        h->plan.spectral ? "spectral_solve" : "circulant_solve_kernel", h->plan.nconv, h->plan.blocks,
        h->plan.nodes_per_block);
    if (k < 0 || size_t(k) >= sizeof(tmp)) return std::string();
    std::string s(tmp);
    if (layout) {
        k = std::snprintf(
            tmp, sizeof(tmp),
            ", \"layout\": {\"Ns\": %lld, \"Nm\": %lld, \"Nq\": %lld, \"stride_t\": %lld, \"hist_stride\": %lld, "
            "\"table_stride\": %lld, \"table_sx\": %d, \"row_step\": %d, \"partial_rows\": %d}, "
            "\"staged_tpn\": %d, \"solve_smem\": %zu, \"solve_why\": \"%s\", "
            "\"adjoint\": {\"ok\": %d, \"threads\": %d, \"grid_x\": %d, \"grid_y\": %d, \"chunk\": %d}}",
            p.Ns, p.Nm, p.Nq, p.stride_t, p.hist_stride, p.table_stride, p.table_sx, p.row_step,
            std::max(h->shape.vblocks, h->staged.ok ? h->staged.ctas : 0), h->staged.tpn, h->plan.smem,
            h->solve_ok ? "" : h->solve_why.c_str(), int(h->aplan.ok), h->aplan.threads, h->aplan.grid_x,
            h->aplan.grid_y, h->aplan.chunk);
        if (k < 0 || size_t(k) >= sizeof(tmp)) return std::string();
        s.pop_back();  // the closing brace
        s += tmp;
    }
    return s;
}

int copy_out(const std::string &s, char *buf, size_t len, const char *who)
{
    if (s.empty()) return fail(nullptr, NUFI_ERR_INVALID, who);
    std::snprintf(buf, len, "%s", s.c_str());
    return s.size() < len ? NUFI_OK : fail(nullptr, NUFI_ERR_RANGE, std::string(who) + ": buffer too small");
}

}  // namespace

extern "C" {

int nufi_describe(const nufi_handle *h, char *buf, size_t len)
{
    if (!h || !buf || len == 0) return fail(nullptr, NUFI_ERR_INVALID, "null argument");
    return copy_out(plan_json(h, false), buf, len, "describe");
}

int nufi_plan(const nufi_config *cfg, int sms, char *buf, size_t len)
{
    return nufi_plan_ex(cfg, nullptr, sms, buf, len);
}

int nufi_plan_ex(const nufi_config *cfg, const nufi_options *opt, int sms, char *buf, size_t len)
{
    if (!buf || len == 0) return fail(nullptr, NUFI_ERR_INVALID, "nufi_plan: null argument");
    if (sms < 1 || sms > 4096) return fail(nullptr, NUFI_ERR_INVALID, "nufi_plan: sms outside [1, 4096]");
    std::string why;
    int st = validate(cfg, why);
    if (st) return fail(nullptr, st, "nufi_plan: " + why);
    nufi_handle h;  // planning only: no stream, no device memory
    if ((st = validate_options(opt, h.opt, why))) return fail(nullptr, st, "nufi_plan: " + why);
    h.cfg = *cfg;
    h.p = make_problem(*cfg);
    h.p.split_plain_kick = h.opt.split_plain_kick;
    h.fp64_table = h.p.precision == NUFI_PREC_FP64 && fp64_table_supported(h.p, cfg->Nt);
    plan_traces(h.p, sms, h.opt, h.shape, h.staged);
    if (h.p.dim == 1 && phase_wraps(h.p) && !h.staged.ok)
        return fail(nullptr, NUFI_ERR_UNSUPPORTED,
                    "nufi_plan: k (x_max - x_min) not a multiple of 2 pi needs the staged FP32-split trace");
    h.solve_ok = solve_geometry(h.p, h.plan, h.solve_why);
    h.persist = plan_persistent(h.p, h.staged, h.plan, h.solve_ok, sms, h.opt);
    h.aplan = adjoint_plan_1d(h.p);
    return copy_out(plan_json(&h, true), buf, len, "nufi_plan");
}

int nufi_solve_kernels(const nufi_config *cfg, double *kernels, int64_t len, int32_t *nconv)
{
    std::string why;
    int st = validate(cfg, why);
    if (st) return fail(nullptr, st, "nufi_solve_kernels: " + why);
    const Problem p = make_problem(*cfg);
    SolvePlan geom;
    if (!solve_geometry(p, geom, why)) return fail(nullptr, NUFI_ERR_UNSUPPORTED, "nufi_solve_kernels: " + why);
    if (nconv) *nconv = geom.nconv;
    if (!kernels) return NUFI_OK;  // size query
    if (len < geom.nconv * p.Ns)
        return fail(nullptr, NUFI_ERR_RANGE, "nufi_solve_kernels: len below nconv * Ns");
    const std::vector<double> g = solve_green(p, geom.nconv);
    std::memcpy(kernels, g.data(), g.size() * sizeof(double));
    return NUFI_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches of 1D instances (batch_1d.cu): one handle per instance for its
// buffers, the batch for the unit maps, the autotuned launch shapes and
// the CUDA graphs of the whole forward and backward.
// ---------------------------------------------------------------------------
struct nufi_batch {
    int device = 0;
    nufi_options opt{};
    cudaStream_t stream = nullptr;
    int precision = 0;
    std::vector<nufi_handle *> inst;
    std::vector<BatchInst> hi;  // host copies of the descriptors
    BatchInst *d_inst = nullptr;
    int *unit_inst = nullptr, *node_inst = nullptr, *solve_inst = nullptr, *adj_unit_inst = nullptr;
    double *theta_acc = nullptr, *grad = nullptr;
    unsigned *err = nullptr;
    BatchLaunch L;
    int maxNt = 0;
    long long point_steps = 0;
    cudaGraphExec_t fwd = nullptr, bwd = nullptr;
    bool forward_done = false;
    // FP32-split forward as one cooperative launch (batch_run_split_kernel)
    // when the autotuner found it faster: its CTAs (0: per-step launches)
    int run_ctas = 0;
    unsigned *run_sync = nullptr;
    std::string last_error, tune;
    std::vector<void *> allocations;
};

namespace {

int bfail(nufi_batch *b, int code, const std::string &msg)
{
    if (b) b->last_error = msg;
    g_last_error = msg;
    return code;
}

int bcuda(nufi_batch *b, cudaError_t e, const char *where)
{
    return bfail(b, NUFI_ERR_CUDA, std::string(where) + ": " + cudaGetErrorName(e) + ": " + cudaGetErrorString(e));
}

template <typename T>
cudaError_t balloc(nufi_batch *b, T **ptr, size_t count)
{
    void *p = nullptr;
    if (count > SIZE_MAX / sizeof(T)) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(count * sizeof(T), 16));
    if (e != cudaSuccess) return e;
    b->allocations.push_back(p);
    *ptr = static_cast<T *>(p);
    return cudaSuccess;
}

void batch_release(nufi_batch *b)
{
    if (b->fwd) cudaGraphExecDestroy(b->fwd);
    if (b->bwd) cudaGraphExecDestroy(b->bwd);
    b->fwd = b->bwd = nullptr;
    for (void *p : b->allocations) cudaFree(p);
    b->allocations.clear();
    for (nufi_handle *h : b->inst) nufi_destroy(h);
    b->inst.clear();
    if (b->stream) cudaStreamDestroy(b->stream);
    b->stream = nullptr;
}

int units_of(const nufi_handle *h, int ppt)
{
    const int tpn = 256 / h->p.N[0];
    return int((h->p.Nm + (long long)tpn * ppt - 1) / ((long long)tpn * ppt));
}

// Forward units for `ppt` chains per thread (descriptors and map uploaded).
int batch_set_units(nufi_batch *b, int ppt, bool adjoint)
{
    std::vector<int> map;
    for (size_t i = 0; i < b->inst.size(); ++i) {
        const int u = units_of(b->inst[i], ppt);
        if (adjoint) {
            b->hi[i].adj_unit_begin = int(map.size());
            b->hi[i].adj_units = u;
        } else {
            b->hi[i].unit_begin = int(map.size());
            b->hi[i].units = u;
        }
        map.insert(map.end(), size_t(u), int(i));
    }
    int *dst = adjoint ? b->adj_unit_inst : b->unit_inst;
    cudaError_t e = cudaMemcpy(dst, map.data(), map.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_inst, b->hi.data(), b->hi.size() * sizeof(BatchInst), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return bcuda(b, e, "batch maps");
    if (adjoint) {
        b->L.adj_ppt = ppt;
        b->L.adj_units = int(map.size());
    } else {
        b->L.ppt = ppt;
        b->L.units = int(map.size());
    }
    return NUFI_OK;
}

// Event time (ms) of `reps` runs of fn on the batch stream after one warm-up.
template <typename F>
float batch_time(nufi_batch *b, F fn, int reps)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    if (fn() != cudaSuccess) return -1;
    cudaEventRecord(e0, b->stream);
    for (int r = 0; r < reps; ++r)
        if (fn() != cudaSuccess) return -1;
    cudaEventRecord(e1, b->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms / reps;
}

// The autotuner: times the candidate launch shapes of the batched trace
// (chains per thread, slabs per ring chunk) at a mid-run step and of the
// adjoint trace (chains per thread), keeps the fastest.  The option
// batch_no_autotune keeps the defaults.
int batch_autotune(nufi_batch *b)
{
    const bool tune = !b->opt.batch_no_autotune;
    const int n_t = std::max(1, b->maxNt / 2);
    size_t ts_max = 0;
    for (nufi_handle *h : b->inst) ts_max = std::max<size_t>(ts_max, size_t(h->p.table_stride));
    std::string log = "{\"trace\": [";
    struct Cand { int ppt, S; };
    std::vector<Cand> cands;
    if (b->precision == NUFI_PREC_FP32_SPLIT) {
        for (int ppt : {2, 4, 8})
            for (int S : {4, 8, 16}) cands.push_back({ppt, S});
    } else {
        for (int ppt : {1, 2, 4}) cands.push_back({ppt, 0});
    }
    if (!tune) cands = {b->precision == NUFI_PREC_FP32_SPLIT ? Cand{4, 8} : Cand{2, 0}};
    float best = -1;
    Cand bc = cands[0];
    for (size_t c = 0; c < cands.size(); ++c) {
        int st = batch_set_units(b, cands[c].ppt, false);
        if (st) return st;
        b->L.slabs_per_chunk = std::max(1, cands[c].S);
        b->L.smem = size_t(kRingSlots) * b->L.slabs_per_chunk * ts_max * sizeof(float);
        float ms = tune ? batch_time(b, [&] { return launch_batch_trace(b->L, n_t, b->stream); }, 2) : 0.0f;
        if (ms < 0) return bcuda(b, cudaGetLastError(), "autotune trace");
        char item[128];
        std::snprintf(item, sizeof(item), "%s{\"ppt\": %d, \"slabs_per_chunk\": %d, \"ms\": %.4f}", c ? ", " : "",
                      cands[c].ppt, cands[c].S, ms);
        log += item;
        if (best < 0 || ms < best) {
            best = ms;
            bc = cands[c];
        }
    }
    int st = batch_set_units(b, bc.ppt, false);
    if (st) return st;
    b->L.slabs_per_chunk = std::max(1, bc.S);
    b->L.smem = size_t(kRingSlots) * b->L.slabs_per_chunk * ts_max * sizeof(float);
    // The whole forward as one cooperative launch against the per-step
    // launches, both timed over three mid-run steps (trace, rho, solve).
    int sms0 = 1;
    cudaDeviceGetAttribute(&sms0, cudaDevAttrMultiProcessorCount, b->device);
    const int run_ctas =
        (b->precision == NUFI_PREC_FP32_SPLIT && !b->opt.no_persistent) ? batch_run_ctas(b->L, sms0) : 0;
    {
        const int n_a = n_t, n_b = std::min(b->maxNt, n_t + 2);
        float ms_steps = 0, ms_run = -1;
        if (tune && run_ctas > 0) {
            ms_steps = batch_time(b, [&] {
                cudaError_t e = cudaSuccess;
                for (int n = n_a; n <= n_b && e == cudaSuccess; ++n) e = launch_batch_step(b->L, n, b->stream);
                return e;
            }, 1);
            if (ms_steps < 0) return bcuda(b, cudaGetLastError(), "autotune forward steps");
        }
        if (run_ctas > 0) {
            cudaError_t ea = balloc(b, &b->run_sync, 2);
            if (ea != cudaSuccess) return bcuda(b, ea, "cudaMalloc");
            ms_run = batch_time(b, [&] { return launch_batch_run(b->L, run_ctas, n_a, n_b, b->run_sync, b->stream); },
                                1);
            if (ms_run < 0) {  // the cooperative launch did not run here: keep the per-step launches
                cudaGetLastError();
                ms_run = -1;
            }
        }
        b->run_ctas = (run_ctas > 0 && ms_run >= 0 && (!tune || ms_run <= ms_steps)) ? run_ctas : 0;
        char item[256];
        std::snprintf(item, sizeof(item),
                      "], \"forward\": {\"per_step_launches_ms\": %.4f, \"one_launch_ms\": %.4f, "
                      "\"one_launch_ctas\": %d, \"steps\": [%d, %d], \"chosen\": \"%s\"}",
                      ms_steps, ms_run, run_ctas, n_a, n_b,
                      b->run_ctas ? "one cooperative launch" : "graph of per-step launches");
        log += item;
    }
    log += ", \"adjoint\": [";
    const bool split = b->precision == NUFI_PREC_FP32_SPLIT;
    std::vector<int> acands = tune ? (split ? std::vector<int>{2, 4} : std::vector<int>{1, 2, 4})
                                   : std::vector<int>{split ? 4 : 2};
    // the option batch_adjoint_ppt = k fixes the adjoint's chains per thread
    if (const int k = b->opt.batch_adjoint_ppt) {
        if (split ? (k == 2 || k == 4) : (k == 1 || k == 2 || k == 4)) acands = {k};
    }
    // FP32-split adjoint: a persistent grid (CTAs per SM from the occupancy
    // of each candidate) and one checkpoint area per CTA; its units are
    // kAdjThreads threads x ppt chains
    auto set_adj = [&](int ppt) {
        if (!split) return batch_set_units(b, ppt, true);
        const int r = batch_set_units(b, ppt * (kAdjThreads / kBatchMaxN), true);
        b->L.adj_ppt = ppt;
        return r;
    };
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    b->L.max_chunks = (b->maxNt + kAdjChunk - 1) / kAdjChunk;
    auto split_grid = [&](int ppt) {
        const int per_sm = std::max(1, adjoint_split_ctas_per_sm(b->L, ppt));
        return std::min(b->L.adj_units, per_sm * std::max(1, sms));
    };
    if (split) {
        size_t need = 0;
        for (int ppt : acands) {
            if ((st = set_adj(ppt))) return st;
            need = std::max(need, size_t(split_grid(ppt)) * b->L.max_chunks * 4 * kAdjThreads * ppt);
        }
        cudaError_t ea = balloc(b, &b->L.ckpt, need);
        if (ea != cudaSuccess) return bcuda(b, ea, "cudaMalloc");
    }
    float abest = -1;
    int abc = acands[0];
    for (size_t c = 0; c < acands.size(); ++c) {
        st = set_adj(acands[c]);
        if (st) return st;
        if (split) b->L.adj_grid = split_grid(acands[c]);
        float ms = tune ? batch_time(b, [&] { return launch_batch_adjoint_step(b->L, n_t, b->stream); }, 1) : 0.0f;
        if (ms < 0) return bcuda(b, cudaGetLastError(), "autotune adjoint");
        char item[96];
        std::snprintf(item, sizeof(item), "%s{\"ppt\": %d, \"ms\": %.4f}", c ? ", " : "", acands[c], ms);
        log += item;
        if (abest < 0 || ms < abest) {
            abest = ms;
            abc = acands[c];
        }
    }
    st = set_adj(abc);
    if (st) return st;
    if (split) b->L.adj_grid = split_grid(abc);
    char tail[160];
    std::snprintf(tail, sizeof(tail), "], \"chosen\": {\"ppt\": %d, \"slabs_per_chunk\": %d, \"adjoint_ppt\": %d, "
                  "\"tuned_at_step\": %d}}", b->L.ppt, b->L.slabs_per_chunk, b->L.adj_ppt, n_t);
    log += tail;
    b->tune = log;
    // the tuning runs wrote into the adjoint scratch and the error word
    cudaMemsetAsync(b->err, 0, sizeof(unsigned), b->stream);
    cudaError_t e = cudaStreamSynchronize(b->stream);
    return e == cudaSuccess ? NUFI_OK : bcuda(b, e, "autotune");
}

int batch_check(nufi_batch *b)
{
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "batch");
    unsigned flags = 0;
    if ((e = cudaMemcpy(&flags, b->err, sizeof(unsigned), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return bcuda(b, e, "batch flags");
    if (flags) {
        cudaMemset(b->err, 0, sizeof(unsigned));
        return bfail(b, NUFI_ERR_DEVICE, "batch: device check failed (flags " + std::to_string(flags) + ")");
    }
    return NUFI_OK;
}

template <typename F>
int capture(nufi_batch *b, cudaGraphExec_t *exec, F body)
{
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return bcuda(b, e, "begin capture");
    cudaError_t eb = body();
    e = cudaStreamEndCapture(b->stream, &g);
    if (eb != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bcuda(b, eb, "batch launch");
    }
    if (e != cudaSuccess) return bcuda(b, e, "end capture");
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    return e == cudaSuccess ? NUFI_OK : bcuda(b, e, "graph instantiate");
}

}  // namespace

extern "C" {

int nufi_batch_create(const nufi_config *cfgs, int32_t count, int device, nufi_batch **out)
{
    return nufi_batch_create_ex(cfgs, count, nullptr, device, out);
}

int nufi_batch_create_ex(const nufi_config *cfgs, int32_t count, const nufi_options *opt, int device,
                         nufi_batch **out)
{
    if (!out || !cfgs || count <= 0) return bfail(nullptr, NUFI_ERR_INVALID, "nufi_batch_create: bad arguments");
    *out = nullptr;
    nufi_options o{};
    {
        std::string why;
        const int st = validate_options(opt, o, why);
        if (st) return bfail(nullptr, st, "nufi_batch_create: " + why);
    }
    for (int32_t i = 0; i < count; ++i) {
        const nufi_config &c = cfgs[i];
        if (c.dim != 1 || c.order != 4 || c.precision != cfgs[0].precision)
            return bfail(nullptr, NUFI_ERR_UNSUPPORTED, "nufi_batch_create: 1D, order 4, one precision per batch");
        if (c.precision == NUFI_PREC_FP32_SPLIT && !phase_is_periodic(c.f0_params[1], c.x_max[0] - c.x_min[0]))
            return bfail(nullptr, NUFI_ERR_UNSUPPORTED,
                         "nufi_batch_create: FP32-split instances need k (x_max - x_min) a multiple of 2 pi");
        if (c.Nx[0] < 1 || c.Nx[0] > kBatchMaxN || kBatchMaxN % c.Nx[0] != 0)
            return bfail(nullptr, NUFI_ERR_UNSUPPORTED, "nufi_batch_create: Nx must divide 256");
    }
    std::unique_ptr<nufi_batch> b(new nufi_batch);
    b->device = device;
    b->opt = o;
    b->precision = cfgs[0].precision;
    auto bail = [&](int code) {
        const std::string msg = b->last_error;
        batch_release(b.get());
        g_last_error = msg;
        return code;
    };
    for (int32_t i = 0; i < count; ++i) {
        nufi_handle *h = nullptr;
        int st = create_handle(&cfgs[i], &o, device, &h, true);
        if (st) {
            b->last_error = "instance " + std::to_string(i) + ": " + g_last_error;
            return bail(st);
        }
        b->inst.push_back(h);
        if (!h->solve_ok) {
            b->last_error = "instance " + std::to_string(i) + ": " + h->solve_why;
            return bail(NUFI_ERR_UNSUPPORTED);
        }
    }
    DeviceGuard g(device);
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(bcuda(b.get(), e, "cudaStreamCreate"));
    long long max_units = 0, max_adj = 0, nodes = 0;
    int solve_blocks = 0, max_P = 0;
    b->hi.resize(size_t(count));
    std::vector<int> node_map, solve_map;
    bool pow2 = true;
    for (int32_t i = 0; i < count; ++i) {
        nufi_handle *h = b->inst[size_t(i)];
        const Problem &p = h->p;
        BatchInst &I = b->hi[size_t(i)];
        std::memset(&I, 0, sizeof(I));
        I.p = p;
        I.hist = h->hist;
        I.tables = h->tables;
        I.nodes = h->nodes;
        I.phase = h->phase;
        I.green = h->plan.green;
        I.rho = h->rho;
        I.energy = h->energy;
        I.Nt = int(h->cfg.Nt);
        I.tpn = kBatchMaxN / p.N[0];
        const int u1 = units_of(h, 1);
        const int nsb = (p.N[0] + 7) / 8;
        if ((e = balloc(b.get(), &I.partial, size_t(u1) * p.N[0])) != cudaSuccess ||
            (e = balloc(b.get(), &I.epart, size_t(nsb))) != cudaSuccess ||
            (e = balloc(b.get(), &I.ecount, 1)) != cudaSuccess ||
            (e = balloc(b.get(), &I.mu, size_t(I.Nt + 1) * p.P[0])) != cudaSuccess ||
            (e = balloc(b.get(), &I.lambda, size_t(p.N[0]))) != cudaSuccess ||
            (b->precision == NUFI_PREC_FP32_SPLIT &&
             ((e = balloc(b.get(), &I.muT, size_t(I.Nt + 1) * 3 * p.N[0])) != cudaSuccess ||
              (e = balloc(b.get(), &I.muS, size_t(I.Nt + 1) * 3 * p.N[0])) != cudaSuccess)))
            return bail(bcuda(b.get(), e, "cudaMalloc"));
        if ((e = cudaMemset(I.ecount, 0, sizeof(unsigned))) != cudaSuccess ||
            (e = cudaMemset(I.lambda, 0, size_t(p.N[0]) * sizeof(double))) != cudaSuccess ||
            (I.muT && (e = cudaMemset(I.muT, 0, size_t(I.Nt + 1) * 3 * p.N[0] * sizeof(double))) != cudaSuccess) ||
            (I.muS && (e = cudaMemset(I.muS, 0, size_t(I.Nt + 1) * 3 * p.N[0] * sizeof(float))) != cudaSuccess) ||
            (e = cudaMemset(I.mu, 0, size_t(I.Nt + 1) * p.P[0] * sizeof(double))) != cudaSuccess)
            return bail(bcuda(b.get(), e, "cudaMemset"));
        I.node_begin = nodes;
        node_map.insert(node_map.end(), size_t(p.N[0]), i);
        nodes += p.N[0];
        I.solve_begin = solve_blocks;
        I.solve_blocks = nsb;
        solve_map.insert(solve_map.end(), size_t(nsb), i);
        solve_blocks += nsb;
        max_units += u1;
        max_adj += u1;
        max_P = std::max(max_P, p.P[0]);
        b->L.ts_max = std::max(b->L.ts_max, int(p.table_stride));
        b->L.max_N = std::max(b->L.max_N, p.N[0]);
        b->maxNt = std::max(b->maxNt, I.Nt);
        b->point_steps += p.Nq * ((long long)I.Nt * (I.Nt + 1) / 2);
        pow2 = pow2 && ((p.N[0] & (p.N[0] - 1)) == 0);
    }
    if ((e = balloc(b.get(), &b->d_inst, size_t(count))) != cudaSuccess ||
        (e = balloc(b.get(), &b->unit_inst, size_t(max_units))) != cudaSuccess ||
        (e = balloc(b.get(), &b->adj_unit_inst, size_t(max_adj))) != cudaSuccess ||
        (e = balloc(b.get(), &b->node_inst, size_t(nodes))) != cudaSuccess ||
        (e = balloc(b.get(), &b->solve_inst, size_t(solve_blocks))) != cudaSuccess ||
        (e = balloc(b.get(), &b->theta_acc, size_t(4 * max_adj))) != cudaSuccess ||
        (e = balloc(b.get(), &b->grad, size_t(4 * count))) != cudaSuccess ||
        (e = balloc(b.get(), &b->err, 1)) != cudaSuccess)
        return bail(bcuda(b.get(), e, "cudaMalloc"));
    if ((e = cudaMemcpy(b->node_inst, node_map.data(), node_map.size() * sizeof(int), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (e = cudaMemcpy(b->solve_inst, solve_map.data(), solve_map.size() * sizeof(int), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (e = cudaMemset(b->err, 0, sizeof(unsigned))) != cudaSuccess)
        return bail(bcuda(b.get(), e, "batch setup"));
    BatchLaunch &L = b->L;
    L.inst = b->d_inst;
    L.unit_inst = b->unit_inst;
    L.node_inst = b->node_inst;
    L.solve_inst = b->solve_inst;
    L.adj_unit_inst = b->adj_unit_inst;
    L.count = count;
    L.precision = b->precision;
    L.pow2 = pow2;
    L.total_nodes = nodes;
    L.solve_blocks = solve_blocks;
    L.max_P = max_P;
    L.adj_chunk = 8;
    L.theta_acc = b->theta_acc;
    L.err = b->err;
    int st = batch_autotune(b.get());
    if (st) return bail(st);
    *out = b.release();
    return NUFI_OK;
}

int nufi_batch_destroy(nufi_batch *b)
{
    if (!b) return NUFI_OK;
    DeviceGuard g(b->device);
    batch_release(b);
    delete b;
    return NUFI_OK;
}

const char *nufi_batch_last_error(const nufi_batch *b) { return b ? b->last_error.c_str() : g_last_error.c_str(); }

int nufi_batch_forward(nufi_batch *b, double *J)
{
    if (!b) return bfail(nullptr, NUFI_ERR_INVALID, "null batch");
    DeviceGuard g(b->device);
    if (!b->fwd) {
        int st = capture(b, &b->fwd, [&] {
            if (b->run_ctas > 0)  // the whole forward: one cooperative launch
                return launch_batch_run(b->L, b->run_ctas, 0, b->maxNt, b->run_sync, b->stream);
            cudaError_t e = cudaSuccess;
            for (int n = 0; n <= b->maxNt && e == cudaSuccess; ++n) e = launch_batch_step(b->L, n, b->stream);
            return e;
        });
        if (st) return st;
    }
    cudaError_t e = cudaGraphLaunch(b->fwd, b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "graph launch");
    int st = batch_check(b);
    if (st) return st;
    for (nufi_handle *h : b->inst) mark_steps(h, 0, h->cfg.Nt, true);
    b->forward_done = true;
    if (J) {
        for (size_t i = 0; i < b->inst.size(); ++i) {
            nufi_handle *h = b->inst[i];
            std::vector<double> w(size_t(h->cfg.Nt + 1));
            e = cudaMemcpy(w.data(), h->energy, w.size() * sizeof(double), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return bcuda(b, e, "energy download");
            double s = 0;
            for (double v : w) s += v;
            J[i] = 2.0 * h->cfg.dt * s;
        }
    }
    return NUFI_OK;
}

int nufi_batch_backward(nufi_batch *b, double *grad)
{
    if (!b || !grad) return bfail(b, NUFI_ERR_INVALID, "null argument");
    if (!b->forward_done) return bfail(b, NUFI_ERR_RANGE, "batch backward: run the forward first");
    if (b->precision == NUFI_PREC_FP32_SPLIT && !b->L.pow2)
        return bfail(b, NUFI_ERR_UNSUPPORTED, "batch backward (FP32-split): Nx must be powers of two");
    DeviceGuard g(b->device);
    if (!b->bwd) {
        int st = capture(b, &b->bwd, [&] {
            cudaError_t e = cudaSuccess;
            for (const BatchInst &I : b->hi)
                if (e == cudaSuccess)
                    e = I.muT ? cudaMemsetAsync(I.muT, 0, size_t(I.Nt + 1) * 3 * I.p.N[0] * sizeof(double), b->stream)
                              : cudaMemsetAsync(I.mu, 0, size_t(I.Nt + 1) * I.p.P[0] * sizeof(double), b->stream);
            for (const BatchInst &I : b->hi)
                if (e == cudaSuccess && I.muS)
                    e = cudaMemsetAsync(I.muS, 0, size_t(I.Nt + 1) * 3 * I.p.N[0] * sizeof(float), b->stream);
            if (e == cudaSuccess)
                e = cudaMemsetAsync(b->theta_acc, 0, size_t(4) * b->L.adj_units * sizeof(double), b->stream);
            for (int m = b->maxNt; m >= 0 && e == cudaSuccess; --m) e = launch_batch_adjoint_step(b->L, m, b->stream);
            if (e == cudaSuccess) e = launch_batch_theta_reduce(b->L, b->grad, b->stream);
            return e;
        });
        if (st) return st;
    }
    cudaError_t e = cudaGraphLaunch(b->bwd, b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "graph launch");
    e = cudaMemcpyAsync(grad, b->grad, size_t(4) * b->L.count * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "grad download");
    return batch_check(b);
}

int nufi_batch_energy(nufi_batch *b, int32_t i, double *energy)
{
    if (!b || !energy) return bfail(b, NUFI_ERR_INVALID, "null argument");
    if (i < 0 || i >= b->L.count) return bfail(b, NUFI_ERR_RANGE, "instance out of range");
    DeviceGuard g(b->device);
    nufi_handle *h = b->inst[size_t(i)];
    cudaError_t e = cudaMemcpy(energy, h->energy, size_t(h->cfg.Nt + 1) * sizeof(double), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? NUFI_OK : bcuda(b, e, "energy download");
}

int nufi_batch_stream(const nufi_batch *b, void **stream)
{
    if (!b || !stream) return bfail(nullptr, NUFI_ERR_INVALID, "null argument");
    *stream = b->stream;
    return NUFI_OK;
}

int nufi_batch_describe(const nufi_batch *b, char *buf, size_t len)
{
    if (!b || !buf || len == 0) return bfail(nullptr, NUFI_ERR_INVALID, "null argument");
    const std::string s = "{\"instances\": " + std::to_string(b->L.count) + ", \"forward_launch\": \"" +
                          (b->run_ctas ? "batch_run_split_kernel (one cooperative launch)"
                                       : "graph of per-step launches") +
                          "\", \"forward_ctas\": " + std::to_string(b->run_ctas) + ", \"units\": " +
                          std::to_string(b->L.units) + ", \"adjoint_units\": " + std::to_string(b->L.adj_units) +
                          ", \"solve_blocks\": " + std::to_string(b->L.solve_blocks) + ", \"max_Nt\": " +
                          std::to_string(b->maxNt) + ", \"point_steps\": " + std::to_string(b->point_steps) +
                          ", \"autotune\": " + b->tune + "}";
    std::snprintf(buf, len, "%s", s.c_str());
    return s.size() < len ? NUFI_OK : bfail(nullptr, NUFI_ERR_RANGE, "describe: buffer too small");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free rho (nufi_compute_rho_noalloc).
//
// For callers that must not allocate device memory: a plugin whose host
// framework owns all device memory through its own pool and forbids direct
// allocation, or a real-time loop that reserves its device memory up front
// because cudaMalloc can synchronise the device and take unbounded time.
// The caller passes the coefficient history and rho as device
// buffers; the trace's scratch (per-block partial sums and an error word)
// lives in the file-scope array below, which every GPU that loads
// this library holds until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;  // 8 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_addr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on the current device, looked up
// once per device.  (In host code the symbol's name is only a host-side
// stand-in; a kernel must be given this address instead.)
int noalloc_scratch(int dev, unsigned char **out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_addr[dev] = static_cast<unsigned char *>(ptr);
    }
    *out = g_noalloc_addr[dev];
    return NUFI_OK;
}

}  // namespace

extern "C" int nufi_compute_rho_noalloc(const nufi_config *cfg, int64_t n, const double *hist, int64_t hist_stride,
                                        int64_t q_begin, int64_t q_end, double *rho, void *stream)
{
    std::string why;
    int st = validate(cfg, why);
    if (st) return fail(nullptr, st, "nufi_compute_rho_noalloc: " + why);
    if (cfg->precision != NUFI_PREC_FP64)
        return fail(nullptr, NUFI_ERR_UNSUPPORTED, "nufi_compute_rho_noalloc: FP64 plain form only");
    if (!hist || !rho) return fail(nullptr, NUFI_ERR_INVALID, "nufi_compute_rho_noalloc: null buffer");
    Problem p = make_problem(*cfg);
    if (hist_stride < p.stride_t)
        return fail(nullptr, NUFI_ERR_INVALID, "nufi_compute_rho_noalloc: hist_stride smaller than one slab");
    // the kernels address slab k at hist + k * hist_stride in 64-bit
    // integers: the history's extent is held to the bound nufi_create uses
    if ((long double)(cfg->Nt + 1) * (long double)hist_stride * 8 > (long double)(1ULL << 50))
        return fail(nullptr, NUFI_ERR_RANGE, "nufi_compute_rho_noalloc: history above 2^50 bytes");
    p.hist_stride = hist_stride;
    if (n < 0 || n > cfg->Nt) return fail(nullptr, NUFI_ERR_RANGE, "nufi_compute_rho_noalloc: Time-step out of range.");
    if (q_begin < 0 || q_end < q_begin || q_end > p.Nq)
        return fail(nullptr, NUFI_ERR_RANGE, "nufi_compute_rho_noalloc: quadrature range outside [0, Nq]");
    if (q_begin == q_end) return NUFI_OK;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(nullptr, NUFI_ERR_INVALID, "nufi_compute_rho_noalloc: device id");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    LaunchShape shape = choose_shape(p, sms > 0 ? sms : 1);
    // Scratch layout: [error word | pad to 256 B][partial sums]
    const size_t off_partial = 256;
    auto need = [&](const LaunchShape &sh) { return off_partial + size_t(sh.vblocks) * size_t(p.Ns) * sizeof(double); };
    if (need(shape) > kNoAllocScratchBytes) {
        // fewest velocity blocks: 4 warps x 4 points per thread
        shape.warps = 4;
        shape.ppt = 4;
        shape.vblocks = int((p.Nm + 15) / 16);
    }
    if (need(shape) > kNoAllocScratchBytes)
        return fail(nullptr, NUFI_ERR_RANGE,
                    "nufi_compute_rho_noalloc: needs " + std::to_string(need(shape)) +
                        " bytes of scratch; the allocation-free entry point holds " +
                        std::to_string(kNoAllocScratchBytes) + " (about Nm * Ns / 16 * 8 bytes must fit)");
    unsigned char *base = nullptr;
    if ((st = noalloc_scratch(dev, &base))) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The previous call's contents stay in the array: the error word must
    // start at zero (the partial sums are overwritten before they are read).
    if ((e = cudaMemsetAsync(base, 0, off_partial, s)) != cudaSuccess)
        return cuda_fail(nullptr, e, "cudaMemsetAsync(scratch)");
    double *partial = reinterpret_cast<double *>(base + off_partial);
    int rows = 0;
    e = launch_trace_fp64(p, shape, hist, int(n), q_begin, q_end, 0, partial, &rows,
                          reinterpret_cast<unsigned *>(base), s);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "nufi_compute_rho_noalloc trace launch");
    e = launch_reduce_rho(p, rows, partial, rho, s);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "nufi_compute_rho_noalloc reduce launch");
    return NUFI_OK;
}
