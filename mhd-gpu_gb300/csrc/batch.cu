// batch.cu - host side of the batched ensemble (include/mhdgpu.h,
// mhdgpu_batch_*): work tables, the per-step launch sequence, the block
// schedule and its autotuner, plus the CFL and clock kernels over all boxes.
// The sweep kernels are in batch_kernel.cuh (instantiated per math policy in
// batch_faithful.cu and batch_fast.cu).
#include <cuda_runtime.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "batch_kernel.cuh"
#include "profiler.cuh"
#include "tunecache.h"

namespace mhd {

// CFL over every box: items are (box, chunk of kCflChunk cells) through a
// prefix table; each CTA reduces its chunk and folds it into the box's word.
constexpr int kCflThreads = 256;
constexpr int kCflChunk = kCflThreads * 16;

struct CflWork {
    const BoxDesc *box;
    const long long *start;   // nbox + 1 prefix sums of chunk counts
    int nbox, mode;
};

__global__ void __launch_bounds__(kCflThreads)
batch_cfl_kernel(CflWork w)
{
    const long long total = w.start[w.nbox];
    for (long long it = blockIdx.x; it < total; it += gridDim.x) {
        int lo = 0, hi = w.nbox - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (w.start[mid] <= it) lo = mid;
            else hi = mid - 1;
        }
        const BoxDesc d = w.box[lo];
        const long long ncell = (long long)d.nx * d.ny * d.nz;
        const long long c0 = (it - w.start[lo]) * kCflChunk;
        const long long c1 = min(c0 + kCflChunk, ncell);
        float cl = 0.0f;
        for (long long c = c0 + threadIdx.x; c < c1; c += blockDim.x)
            cl = fmaxf(cl, cfl_cell_speed(d.u, d.b, d.nx, d.ny, d.nz, w.mode, c));
        cfl_block_max(cl, &d.clk->cmax);
    }
}

// Each box's CFL word cleared before a reduction pass: the state may have
// changed since the last step folded its speed into the word.
__global__ void batch_cmax_clear_kernel(const BoxDesc *box, int nbox)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nbox) box[i].clk->cmax = 0u;
}

// One clock tick per box, and the sweeps' claim and completion counters
// cleared for the step.
__global__ void batch_clock_kernel(const BoxDesc *box, const float *tf, int nbox, double cfl_number,
                                   unsigned *ctr, int nctr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (int c = i; c < nctr; c += gridDim.x * blockDim.x) ctr[c] = 0u;
    if (i < nbox) clock_tick(box[i].clk, cfl_number, tf[i], nullptr);
}

}  // namespace mhd

using namespace mhd;

namespace {

constexpr int kSweepAxis[6] = {0, 1, 2, 2, 1, 0};
// parts of mhdgpu_batch_run_host's pipeline (the upload of one part overlaps
// the steps of the parts before it, their downloads the steps after it)
constexpr int kHostParts = 4;
constexpr int kSweepFluidFirst[6] = {1, 1, 1, 0, 0, 0};
constexpr int kThreadChoices[3] = {64, 128, 256};

}  // namespace

// one persistent launch: the boxes of one team class in one sweep
struct BatchGroup {
    int sweep = 0, cls = 0, nb = 0;
    std::vector<int> boxes;       // batch indices of the group's boxes
    size_t off_args = 0;          // first entry in d_fa / d_aa
    size_t off_start = 0;         // first entry in d_start (3 nb + 1)
    size_t off_group = 0;         // first entry in d_group (3 nb)
    size_t off_ctr = 0;           // claim word, then 3 nb completion words, in d_ctr
    long long cells = 0, items = 0;
    size_t smem = 0;
    int grid = 1;
    int threads = 256;            // CTA size of the launch
};

struct mhdgpu_batch {
    int nbox = 0;
    int device = 0, num_sms = 0;
    double cfl_number = 0.0;
    int cfl_mode = MHD_CFL_C;
    std::vector<BoxDesc> box;
    BoxDesc *d_box = nullptr;
    mhdgpu_clock *d_clk = nullptr;
    float *d_scr = nullptr;
    float *d_tf = nullptr;
    std::vector<BatchGroup> groups;     // ordered by sweep
    int gbegin[7] = {};                 // groups of sweep s: [gbegin[s], gbegin[s+1])
    std::vector<FluidxArgs> fa;         // 6 * nbox entries (host: they travel in the launches)
    std::vector<AdvectArgs> aa;
    long long *d_start = nullptr;
    int *d_group = nullptr;
    unsigned *d_ctr = nullptr;          // the groups' counters, then the abort word
    int nctr = 0;
    unsigned *d_abort = nullptr;
    long long *d_cfl_start = nullptr;   // nbox + 1
    long long cfl_total = 0;
    int threads[3] = {256, 256, 256};
    int cps[3] = {8, 8, 8};             // CTAs per SM cap (the occupancy limits it further)
    unsigned stall_extra = 0;           // mhdgpu_batch_inject_stall
    bool folded = false;                // a step was enqueued: the clocks hold the folded CFL speeds
    ClassWork work{};                   // parameter block of one launch (filled per launch)
    cudaStream_t side[kBatchClasses] = {};
    cudaEvent_t fork = nullptr, join[kBatchClasses] = {};
    std::vector<float> tf_host;         // each box's end time (0: none)
    // mhdgpu_batch_run_host's pipeline: parts of the boxes (views that share
    // this handle's states, scratch, clock records and abort word), built on
    // first use and dropped when the schedule changes
    std::vector<mhdgpu_batch *> parts;
    std::vector<std::vector<int>> part_boxes;
    cudaEvent_t up[kHostParts] = {};

    ~mhdgpu_batch()
    {
        drop_parts();
        cudaFree(d_box); cudaFree(d_clk); cudaFree(d_scr); cudaFree(d_tf);
        cudaFree(d_ctr); cudaFree(d_start); cudaFree(d_group); cudaFree(d_cfl_start);
        for (int i = 0; i < kBatchClasses; ++i) {
            if (side[i]) cudaStreamDestroy(side[i]);
            if (join[i]) cudaEventDestroy(join[i]);
        }
        if (fork) cudaEventDestroy(fork);
        for (int i = 0; i < kHostParts; ++i)
            if (up[i]) cudaEventDestroy(up[i]);
    }
    void drop_parts()
    {
        for (mhdgpu_batch *p : parts) delete p;
        parts.clear();
        part_boxes.clear();
    }
};

namespace {

thread_local char g_berr[256];

int bfail(int st, const char *msg)
{
    set_last_error(msg);
    return st;
}

int bcuda(cudaError_t e, const char *where)
{
    snprintf(g_berr, sizeof g_berr, "%s: %s", where, cudaGetErrorString(e));
    set_last_error(g_berr);
    return MHD_ERR_CUDA;
}

#define BCU(call, where)                                      \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return bcuda(e_, where);       \
    } while (0)

bool dims_ok(int nbox, const int *dims)
{
    if (nbox < 1 || nbox > MHD_BATCH_MAX_BOXES || !dims) return false;
    for (int i = 0; i < 3 * nbox; ++i)
        if (dims[i] < 1 || dims[i] > kBatchMaxPencil) return false;
    return true;
}

long long cells_of(const int *d) { return (long long)d[0] * d[1] * d[2]; }

int occupancy(int cls, bool rows, int threads, size_t smem)
{
    switch (math_mode()) {
    case MHD_MATH_FAST: return batch_class_occupancy_fast(cls, rows, threads, smem);
    case MHD_MATH_FP64P: return batch_class_occupancy_p64(cls, rows, threads, smem);
    default: return batch_class_occupancy_faithful(cls, rows, threads, smem);
    }
}

cudaError_t launch_group(const ClassWork &w, int cls, bool rows, int grid, int threads, size_t smem,
                         cudaStream_t s)
{
    switch (math_mode()) {
    case MHD_MATH_FAST: return launch_batch_class_fast(w, cls, rows, grid, threads, smem, s);
    case MHD_MATH_FP64P: return launch_batch_class_p64(w, cls, rows, grid, threads, smem, s);
    default: return launch_batch_class_faithful(w, cls, rows, grid, threads, smem, s);
    }
}

// Groups the boxes of every sweep by team class and lays out the per-group
// tables; sizes only (no device work).  Counter words are reset every step by
// the clock kernel, so their layout may change between steps.
void plan_groups(mhdgpu_batch &bt)
{
    bt.groups.clear();
    size_t off_args = 0, off_start = 0, off_group = 0, off_ctr = 0;
    for (int s = 0; s < 6; ++s) {
        bt.gbegin[s] = (int)bt.groups.size();
        const int axis = kSweepAxis[s];
        // the classes of the sweep, fewest cells first: their launches start in
        // this order (on GB300 the ensemble's step is about 2% faster than
        // with the classes in index order, 1% faster than most cells first)
        std::vector<std::vector<int>> by_class(kBatchClasses);
        std::vector<long long> class_cells(kBatchClasses, 0);
        for (int i = 0; i < bt.nbox; ++i) {
            const BoxDesc &d = bt.box[i];
            const int cls = batch_class(make_view(axis, d.nx, d.ny, d.nz).n);
            by_class[cls].push_back(i);
            class_cells[cls] += (long long)d.nx * d.ny * d.nz;
        }
        std::vector<int> order(kBatchClasses);
        for (int c = 0; c < kBatchClasses; ++c) order[c] = c;
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return class_cells[a] < class_cells[b]; });
        for (int cls : order) {
            const std::vector<int> &members = by_class[cls];
            // a launch carries at most kGroupBoxes boxes' arguments
            for (size_t m0 = 0; m0 < members.size(); m0 += kGroupBoxes) {
                BatchGroup g;
                g.sweep = s;
                g.cls = cls;
                const size_t m1 = std::min(members.size(), m0 + (size_t)kGroupBoxes);
                for (size_t m = m0; m < m1; ++m) {
                    const BoxDesc &d = bt.box[members[m]];
                    const Frame f = make_view(axis, d.nx, d.ny, d.nz);
                    g.boxes.push_back(members[m]);
                    g.cells += f.npen * f.n;
                }
                g.nb = (int)g.boxes.size();
                g.off_args = off_args;
                g.off_start = off_start;
                g.off_group = off_group;
                g.off_ctr = off_ctr;
                off_args += g.nb;
                off_start += 3 * g.nb + 1;
                off_group += 3 * g.nb;
                off_ctr += 1 + 3 * g.nb;
                bt.groups.push_back(g);
            }
        }
    }
    bt.gbegin[6] = (int)bt.groups.size();
    bt.nctr = (int)off_ctr;
}

// (re)builds the work tables and the launch shapes for the current schedule;
// synchronous.  The device tables are read by the class kernels of every step
// already enqueued, on whatever stream: the upload waits for the device to
// drain first, so that a step in flight never sees half of a new schedule.
int build_tables(mhdgpu_batch &bt)
{
    std::vector<FluidxArgs> &fa = bt.fa;
    std::vector<AdvectArgs> &aa = bt.aa;
    fa.clear();
    aa.clear();
    std::vector<long long> start;
    std::vector<int> group;
    for (BatchGroup &g : bt.groups) {
        const int axis = kSweepAxis[g.sweep];
        const bool rows = axis != 0;
        // at most 8 pencils per CTA (the row staging's lane layout)
        const int tpp = batch_class_tpp(g.cls);
        const int threads = std::min(bt.threads[axis], 8 * tpp);
        g.threads = threads;
        const int ppc = threads / tpp;
        if (ppc < 1)
            return bfail(MHD_ERR_ARG, "mhdgpu_batch: fewer threads per CTA than a pencil's team "
                                      "(64 for pencils of 65-127 cells other than 96, 128 above 128)");
        std::vector<long long> st(3 * g.nb + 1);
        std::vector<int> gr(3 * g.nb);
        long long acc = 0;
        long long sm = 0;
        for (int slot = 0; slot < 3; ++slot) {
            const int ph = batch_phase(slot, kSweepFluidFirst[g.sweep]);
            for (int b = 0; b < g.nb; ++b) {
                const BoxDesc &d = bt.box[g.boxes[b]];
                const Frame f = make_view(axis, d.nx, d.ny, d.nz);
                int per;
                long long items;
                if (ph == kPhaseB1) {
                    per = kB1ItemCells;
                    items = batch_chunks(f.npen * f.n, per);
                } else {
                    per = std::max(1, kItemCells / (ppc * f.n));
                    items = (batch_tiles(f, ppc, rows) + per - 1) / per;
                }
                st[slot * g.nb + b] = acc;
                gr[slot * g.nb + b] = per;
                acc += items;
                if (slot == 0) {
                    sm = std::max(sm, fx_tile_smem_floats(f.n, ppc, batch_class_cpl(g.cls), batch_class_wpp(g.cls), rows));
                    sm = std::max(sm, ax_tile_smem_floats(f.n, ppc, batch_class_cpl(g.cls), batch_class_wpp(g.cls), rows));
                }
            }
        }
        st[3 * g.nb] = acc;
        if (acc >= (1LL << 31)) return bfail(MHD_ERR_ARG, "mhdgpu_batch: too many work items");
        g.items = acc;
        g.smem = sizeof(float) * (size_t)sm;
        if (g.smem > 227 * 1024) return bfail(MHD_ERR_ARG, "mhdgpu_batch: tile exceeds shared memory");
        start.insert(start.end(), st.begin(), st.end());
        group.insert(group.end(), gr.begin(), gr.end());
        for (int b = 0; b < g.nb; ++b) {
            const BoxDesc &d = bt.box[g.boxes[b]];
            const Frame f = make_view(axis, d.nx, d.ny, d.nz);
            // the step's last sweep (x, fluid last) folds the next step's CFL
            // reduction into the box's clock word
            if (g.sweep == 5)
                fa.push_back(FluidxArgs{d.u, d.u, d.b, &d.clk->dt, &d.clk->health, f, &d.clk->cmax, bt.cfl_mode});
            else
                fa.push_back(FluidxArgs{d.u, d.u, d.b, &d.clk->dt, &d.clk->health, f});
            aa.push_back(make_advect_args(d.b, d.u, &d.clk->dt, d.scr, d.scr + f.npen * f.n, f));
        }
    }
    // grids: every group gets the whole GPU at its kernel's occupancy (capped
    // by the schedule).  The groups of a sweep are launched concurrently, so a
    // group's CTAs take the SMs that the previous group's tail frees; grids
    // sized to a share of the SMs were measured slower (the groups do not run
    // side by side, each then runs on its share alone).
    for (int s = 0; s < 6; ++s) {
        const int axis = kSweepAxis[s];
        for (int gi = bt.gbegin[s]; gi < bt.gbegin[s + 1]; ++gi) {
            BatchGroup &g = bt.groups[gi];
            const int occ = occupancy(g.cls, axis != 0, g.threads, g.smem);
            if (occ < 1) return bfail(MHD_ERR_CUDA, "mhdgpu_batch: a class kernel cannot be resident");
            g.grid = (int)std::max(1LL, std::min((long long)bt.num_sms * std::min(bt.cps[axis], occ), g.items));
        }
    }
    BCU(cudaDeviceSynchronize(), "mhdgpu_batch tables");
    BCU(cudaMemcpy(bt.d_start, start.data(), start.size() * sizeof(long long), cudaMemcpyHostToDevice),
        "mhdgpu_batch tables");
    BCU(cudaMemcpy(bt.d_group, group.data(), group.size() * sizeof(int), cudaMemcpyHostToDevice),
        "mhdgpu_batch tables");
    return MHD_OK;
}

// One step.  With first set the CFL reduction runs as its own pass (on
// cleared words); otherwise the previous step's last sweep has folded it into
// the clock words.
int launch_step(mhdgpu_batch &bt, cudaStream_t s, cudaEvent_t *ev /* 7 events or NULL */, bool first)
{
    const int nb = bt.nbox;
    if (poison_scratch()) {
        // every box's flux scratch filled with NaN: a read before its write shows in the state
        for (int i = 0; i < nb; ++i) {
            const BoxDesc &d = bt.box[i];
            BCU(cudaMemsetAsync(d.scr, 0xFF, 2 * sizeof(float) * (size_t)d.nx * d.ny * d.nz, s),
                "mhdgpu_batch poison");
        }
    }
    {
        ProfScope ps(MHD_KCLASS_CFL, first ? 3 : 1, s);
        if (first) {
            batch_cmax_clear_kernel<<<(nb + 255) / 256, 256, 0, s>>>(bt.d_box, nb);
            BCU(cudaGetLastError(), "mhdgpu_batch_advance cfl");
            CflWork cw{bt.d_box, bt.d_cfl_start, nb, bt.cfl_mode};
            const int g = (int)std::max(1LL, std::min((long long)bt.num_sms * 8, bt.cfl_total));
            batch_cfl_kernel<<<g, kCflThreads, 0, s>>>(cw);
            BCU(cudaGetLastError(), "mhdgpu_batch_advance cfl");
        }
        const int gc = (std::max(nb, bt.nctr) + 255) / 256;
        batch_clock_kernel<<<gc, 256, 0, s>>>(bt.d_box, bt.d_tf, nb, bt.cfl_number, bt.d_ctr, bt.nctr);
        BCU(cudaGetLastError(), "mhdgpu_batch_advance clock");
    }
    for (int sw = 0; sw < 6; ++sw) {
        const int axis = kSweepAxis[sw];
        const int g0 = bt.gbegin[sw], g1 = bt.gbegin[sw + 1];
        if (ev) BCU(cudaEventRecord(ev[sw], s), "mhdgpu_batch event");
        ProfScope ps(MHD_KCLASS_BATCH, g1 - g0, s);
        const bool fan = g1 - g0 > 1;
        if (fan) BCU(cudaEventRecord(bt.fork, s), "mhdgpu_batch fork");
        for (int gi = g0; gi < g1; ++gi) {
            const BatchGroup &g = bt.groups[gi];
            ClassWork &w = bt.work;
            std::copy(bt.fa.begin() + g.off_args, bt.fa.begin() + g.off_args + g.nb, w.fa);
            std::copy(bt.aa.begin() + g.off_args, bt.aa.begin() + g.off_args + g.nb, w.aa);
            w.start = bt.d_start + g.off_start;
            w.group = bt.d_group + g.off_group;
            w.claim = bt.d_ctr + g.off_ctr;
            w.done = bt.d_ctr + g.off_ctr + 1;
            w.abort = bt.d_abort;
            w.nb = g.nb;
            w.fluid_first = kSweepFluidFirst[sw];
            w.stall_extra = gi == 0 ? bt.stall_extra : 0u;
            cudaStream_t gs = s;
            if (fan) {
                gs = bt.side[(gi - g0) % kBatchClasses];
                BCU(cudaStreamWaitEvent(gs, bt.fork, 0), "mhdgpu_batch fork");
            }
            BCU(launch_group(w, g.cls, axis != 0, g.grid, g.threads, g.smem, gs), "mhdgpu_batch_advance sweep");
            if (fan) {
                BCU(cudaEventRecord(bt.join[(gi - g0) % kBatchClasses], gs), "mhdgpu_batch join");
                BCU(cudaStreamWaitEvent(s, bt.join[(gi - g0) % kBatchClasses], 0), "mhdgpu_batch join");
            }
        }
    }
    if (ev) BCU(cudaEventRecord(ev[6], s), "mhdgpu_batch event");
    return MHD_OK;
}

// A part of a handle for the host pipeline: the boxes idx of p with p's
// states, scratch slices, clock records, end times, schedule and abort word,
// and its own work tables, counters, streams and events.
int make_part(const mhdgpu_batch &p, const std::vector<int> &idx, mhdgpu_batch **out)
{
    *out = nullptr;
    const int nbox = (int)idx.size();
    mhdgpu_batch *bt = new mhdgpu_batch;
    bt->nbox = nbox;
    bt->device = p.device;
    bt->num_sms = p.num_sms;
    bt->cfl_number = p.cfl_number;
    bt->cfl_mode = p.cfl_mode;
    std::copy(p.threads, p.threads + 3, bt->threads);
    std::copy(p.cps, p.cps + 3, bt->cps);
    std::vector<long long> cfl_start(nbox + 1);
    std::vector<float> htf(nbox);
    for (int j = 0; j < nbox; ++j) {
        const BoxDesc &d = p.box[idx[j]];
        bt->box.push_back(d);
        htf[j] = p.tf_host[idx[j]];
        cfl_start[j] = bt->cfl_total;
        bt->cfl_total += batch_chunks((long long)d.nx * d.ny * d.nz, kCflChunk);
    }
    cfl_start[nbox] = bt->cfl_total;
    bt->tf_host = htf;
    plan_groups(*bt);
    const size_t ngroups = bt->groups.size();
    cudaError_t e = cudaMalloc(&bt->d_box, nbox * sizeof(BoxDesc));
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_tf, nbox * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_ctr, (bt->nctr + 1) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_start, (18 * (size_t)nbox + ngroups) * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_group, 18 * (size_t)nbox * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_cfl_start, (nbox + 1) * sizeof(long long));
    for (int i = 0; i < kBatchClasses && e == cudaSuccess; ++i) {
        e = cudaStreamCreateWithFlags(&bt->side[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bt->join[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bt->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMemcpy(bt->d_box, bt->box.data(), nbox * sizeof(BoxDesc), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(bt->d_ctr, 0, (bt->nctr + 1) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemcpy(bt->d_tf, htf.data(), nbox * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(bt->d_cfl_start, cfl_start.data(), (nbox + 1) * sizeof(long long), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete bt;
        return bcuda(e, "mhdgpu_batch_run_host parts");
    }
    bt->d_abort = p.d_abort;    // a wait that gives up in a part is the handle's
    const int st = build_tables(*bt);
    if (st != MHD_OK) {
        delete bt;
        return st;
    }
    *out = bt;
    return MHD_OK;
}

// Splits the boxes into min(kHostParts, nbox) parts of about equal cells
// (largest box first, each to the part with the fewest cells).
int build_parts(mhdgpu_batch &bt)
{
    const int np = std::min(kHostParts, bt.nbox);
    std::vector<int> order(bt.nbox);
    for (int i = 0; i < bt.nbox; ++i) order[i] = i;
    auto cells = [&](int i) { return (long long)bt.box[i].nx * bt.box[i].ny * bt.box[i].nz; };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cells(a) > cells(b); });
    std::vector<std::vector<int>> part(np);
    std::vector<long long> load(np, 0);
    for (int i : order) {
        const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        part[k].push_back(i);
        load[k] += cells(i);
    }
    for (int k = 0; k < np; ++k) {
        std::sort(part[k].begin(), part[k].end());
        if (!bt.up[k]) BCU(cudaEventCreateWithFlags(&bt.up[k], cudaEventDisableTiming), "mhdgpu_batch_run_host");
        mhdgpu_batch *q = nullptr;
        const int st = make_part(bt, part[k], &q);
        if (st != MHD_OK) {
            bt.drop_parts();
            return st;
        }
        bt.parts.push_back(q);
        bt.part_boxes.push_back(part[k]);
    }
    return MHD_OK;
}

}  // namespace

extern "C" {

size_t mhdgpu_batch_workspace_bytes(int nbox, const int *dims)
{
    if (!dims_ok(nbox, dims)) return 0;
    long long cells = 0;
    for (int i = 0; i < nbox; ++i) cells += cells_of(dims + 3 * i);
    // upper bounds of the tables: 6 sweeps x (8 classes + a split per 64 boxes)
    const size_t ngroups = 6 * (8 + (size_t)nbox / kGroupBoxes + 1);
    const size_t nctr = ngroups + 18 * (size_t)nbox + 1;
    return sizeof(float) * 2 * (size_t)cells + nbox * (sizeof(BoxDesc) + sizeof(mhdgpu_clock) + sizeof(float)) +
           nctr * sizeof(unsigned) +
           (18 * (size_t)nbox + ngroups + nbox + 1) * sizeof(long long) + 18 * (size_t)nbox * sizeof(int);
}

int mhdgpu_batch_create(mhdgpu_batch **out, int nbox, const int *dims, float *const *d_u,
                        float *const *d_b, double cfl_number, int cfl_mode, const float *tf)
{
    if (!out) return bfail(MHD_ERR_ARG, "mhdgpu_batch_create: null handle pointer");
    *out = nullptr;
    if (!dims_ok(nbox, dims))
        return bfail(MHD_ERR_ARG, "mhdgpu_batch_create: need 1..65536 boxes, each axis 1..MHD_BATCH_MAX_PENCIL");
    if (!d_u || !d_b) return bfail(MHD_ERR_ARG, "mhdgpu_batch_create: null state table");
    for (int i = 0; i < nbox; ++i)
        if (!d_u[i] || !d_b[i]) return bfail(MHD_ERR_ARG, "mhdgpu_batch_create: null box state");
    if (!(cfl_number > 0.0)) return bfail(MHD_ERR_ARG, "mhdgpu_batch_create: cfl_number must be > 0");
    if (cfl_mode != MHD_CFL_C && cfl_mode != MHD_CFL_AVERAGED)
        return bfail(MHD_ERR_ARG, "mhdgpu_batch_create: bad cfl mode");
    mhdgpu_batch *bt = new mhdgpu_batch;
    bt->nbox = nbox;
    bt->cfl_number = cfl_number;
    bt->cfl_mode = cfl_mode;
    cudaError_t e = cudaGetDevice(&bt->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&bt->num_sms, cudaDevAttrMultiProcessorCount, bt->device);
    long long cells = 0;
    std::vector<long long> cfl_start(nbox + 1);
    for (int i = 0; i < nbox; ++i) {
        cfl_start[i] = bt->cfl_total;
        const long long nc = cells_of(dims + 3 * i);
        bt->cfl_total += batch_chunks(nc, kCflChunk);
        cells += nc;
    }
    cfl_start[nbox] = bt->cfl_total;
    std::vector<float> htf(nbox, 0.0f);
    if (tf) std::copy(tf, tf + nbox, htf.begin());
    bt->tf_host = htf;
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_box, nbox * sizeof(BoxDesc));
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_clk, nbox * sizeof(mhdgpu_clock));
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_scr, 2 * sizeof(float) * (size_t)cells);
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_tf, nbox * sizeof(float));
    bt->box.resize(nbox);
    long long off = 0;
    for (int i = 0; i < nbox; ++i) {
        BoxDesc &d = bt->box[i];
        d.u = d_u[i];
        d.b = d_b[i];
        d.scr = bt->d_scr + 2 * off;
        d.clk = bt->d_clk + i;
        d.nx = dims[3 * i];
        d.ny = dims[3 * i + 1];
        d.nz = dims[3 * i + 2];
        d.pad = 0;
        off += cells_of(dims + 3 * i);
    }
    plan_groups(*bt);
    const size_t ngroups = bt->groups.size();
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_ctr, (bt->nctr + 1) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_start, (18 * (size_t)nbox + ngroups) * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_group, 18 * (size_t)nbox * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_cfl_start, (nbox + 1) * sizeof(long long));
    for (int i = 0; i < kBatchClasses && e == cudaSuccess; ++i) {
        e = cudaStreamCreateWithFlags(&bt->side[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bt->join[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bt->fork, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        delete bt;
        return bcuda(e, "mhdgpu_batch_create");
    }
    bt->d_abort = bt->d_ctr + bt->nctr;
    e = cudaMemcpy(bt->d_box, bt->box.data(), nbox * sizeof(BoxDesc), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(bt->d_clk, 0, nbox * sizeof(mhdgpu_clock));
    if (e == cudaSuccess) e = cudaMemset(bt->d_ctr, 0, (bt->nctr + 1) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemcpy(bt->d_tf, htf.data(), nbox * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(bt->d_cfl_start, cfl_start.data(), (nbox + 1) * sizeof(long long), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete bt;
        return bcuda(e, "mhdgpu_batch_create");
    }
    const int st = build_tables(*bt);
    if (st != MHD_OK) {
        delete bt;
        return st;
    }
    *out = bt;
    return MHD_OK;
}

int mhdgpu_batch_destroy(mhdgpu_batch *bt)
{
    if (!bt) return bfail(MHD_ERR_ARG, "mhdgpu_batch_destroy: null handle");
    delete bt;
    return MHD_OK;
}

static int batch_steps(mhdgpu_batch *bt, int nsteps, bool resume, mhdgpu_stream_t stream)
{
    if (!bt) return bfail(MHD_ERR_ARG, resume ? "mhdgpu_batch_resume: null handle" : "mhdgpu_batch_advance: null handle");
    if (nsteps < 0) return bfail(MHD_ERR_ARG, resume ? "mhdgpu_batch_resume: nsteps < 0" : "mhdgpu_batch_advance: nsteps < 0");
    for (int it = 0; it < nsteps; ++it) {
        const int st = launch_step(*bt, (cudaStream_t)stream, nullptr, it == 0 && !(resume && bt->folded));
        if (st) return st;
        bt->folded = true;
    }
    return MHD_OK;
}

int mhdgpu_batch_advance(mhdgpu_batch *bt, int nsteps, mhdgpu_stream_t stream)
{
    return batch_steps(bt, nsteps, false, stream);
}

int mhdgpu_batch_resume(mhdgpu_batch *bt, int nsteps, mhdgpu_stream_t stream)
{
    return batch_steps(bt, nsteps, true, stream);
}

// copies of every box between host and device, spread over the side streams
// (several copy engines at once), forked from and joined back to s
static int batch_copy_host(mhdgpu_batch &bt, float *const *h_u, float *const *h_b, bool to_device,
                           cudaStream_t s)
{
    BCU(cudaEventRecord(bt.fork, s), "mhdgpu_batch_run_host fork");
    const int ns = std::min(bt.nbox, kBatchClasses);
    for (int k = 0; k < ns; ++k) BCU(cudaStreamWaitEvent(bt.side[k], bt.fork, 0), "mhdgpu_batch_run_host fork");
    for (int i = 0; i < bt.nbox; ++i) {
        const BoxDesc &d = bt.box[i];
        const size_t nc = (size_t)d.nx * d.ny * d.nz;
        cudaStream_t cs = bt.side[i % ns];
        if (to_device) {
            BCU(cudaMemcpyAsync(d.u, h_u[i], 5 * nc * sizeof(float), cudaMemcpyHostToDevice, cs), "mhdgpu_batch_run_host upload");
            BCU(cudaMemcpyAsync(d.b, h_b[i], 3 * nc * sizeof(float), cudaMemcpyHostToDevice, cs), "mhdgpu_batch_run_host upload");
        } else {
            BCU(cudaMemcpyAsync(h_u[i], d.u, 5 * nc * sizeof(float), cudaMemcpyDeviceToHost, cs), "mhdgpu_batch_run_host download");
            BCU(cudaMemcpyAsync(h_b[i], d.b, 3 * nc * sizeof(float), cudaMemcpyDeviceToHost, cs), "mhdgpu_batch_run_host download");
        }
    }
    for (int k = 0; k < ns; ++k) {
        BCU(cudaEventRecord(bt.join[k], bt.side[k]), "mhdgpu_batch_run_host join");
        BCU(cudaStreamWaitEvent(s, bt.join[k], 0), "mhdgpu_batch_run_host join");
    }
    return MHD_OK;
}

int mhdgpu_batch_run_host(mhdgpu_batch *bt, float *const *h_u, float *const *h_b, int nsteps,
                          mhdgpu_stream_t stream)
{
    if (!bt || !h_u || !h_b) return bfail(MHD_ERR_ARG, "mhdgpu_batch_run_host: null pointer");
    if (nsteps < 0) return bfail(MHD_ERR_ARG, "mhdgpu_batch_run_host: nsteps < 0");
    for (int i = 0; i < bt->nbox; ++i)
        if (!h_u[i] || !h_b[i]) return bfail(MHD_ERR_ARG, "mhdgpu_batch_run_host: null box buffer");
    cudaStream_t s = (cudaStream_t)stream;
    int st = MHD_OK;
    // the state is written from the host: each part's first step runs the CFL pass
    bt->folded = false;
    if (bt->nbox < 2) {
        st = batch_copy_host(*bt, h_u, h_b, true, s);
        if (st) return st;
        for (int it = 0; it < nsteps; ++it) {
            st = launch_step(*bt, s, nullptr, it == 0);
            if (st) return st;
        }
        st = batch_copy_host(*bt, h_u, h_b, false, s);
        if (st) return st;
    } else {
        // Pipeline over parts of about equal cells, one stream each: part k
        // uploads after part k-1 (the host link is the bound), then steps at
        // once while the later parts upload; its download follows its steps
        // while the later parts still step.
        if (bt->parts.empty() && (st = build_parts(*bt)) != MHD_OK) return st;
        const int np = (int)bt->parts.size();
        BCU(cudaEventRecord(bt->fork, s), "mhdgpu_batch_run_host fork");
        for (int k = 0; k < np; ++k) {
            cudaStream_t cs = bt->side[k];
            BCU(cudaStreamWaitEvent(cs, bt->fork, 0), "mhdgpu_batch_run_host fork");
            if (k > 0) BCU(cudaStreamWaitEvent(cs, bt->up[k - 1], 0), "mhdgpu_batch_run_host chain");
            for (int i : bt->part_boxes[k]) {
                const BoxDesc &d = bt->box[i];
                const size_t nc = (size_t)d.nx * d.ny * d.nz;
                BCU(cudaMemcpyAsync(d.u, h_u[i], 5 * nc * sizeof(float), cudaMemcpyHostToDevice, cs),
                    "mhdgpu_batch_run_host upload");
                BCU(cudaMemcpyAsync(d.b, h_b[i], 3 * nc * sizeof(float), cudaMemcpyHostToDevice, cs),
                    "mhdgpu_batch_run_host upload");
            }
            BCU(cudaEventRecord(bt->up[k], cs), "mhdgpu_batch_run_host chain");
            for (int it = 0; it < nsteps; ++it)
                if ((st = launch_step(*bt->parts[k], cs, nullptr, it == 0)) != MHD_OK) return st;
        }
        // downloads are issued after every part's steps: a copy into pageable
        // memory returns only when done, and must not hold back later parts
        for (int k = 0; k < np; ++k) {
            cudaStream_t cs = bt->side[k];
            for (int i : bt->part_boxes[k]) {
                const BoxDesc &d = bt->box[i];
                const size_t nc = (size_t)d.nx * d.ny * d.nz;
                BCU(cudaMemcpyAsync(h_u[i], d.u, 5 * nc * sizeof(float), cudaMemcpyDeviceToHost, cs),
                    "mhdgpu_batch_run_host download");
                BCU(cudaMemcpyAsync(h_b[i], d.b, 3 * nc * sizeof(float), cudaMemcpyDeviceToHost, cs),
                    "mhdgpu_batch_run_host download");
            }
            BCU(cudaEventRecord(bt->join[k], cs), "mhdgpu_batch_run_host join");
            BCU(cudaStreamWaitEvent(s, bt->join[k], 0), "mhdgpu_batch_run_host join");
        }
    }
    // the clocks now hold the last step's folded CFL speeds
    bt->folded = nsteps > 0;
    BCU(cudaStreamSynchronize(s), "mhdgpu_batch_run_host");
    return MHD_OK;
}

int mhdgpu_batch_read_clocks(mhdgpu_batch *bt, mhdgpu_clock *clocks, mhdgpu_stream_t stream)
{
    if (!bt || !clocks) return bfail(MHD_ERR_ARG, "mhdgpu_batch_read_clocks: null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    unsigned abort_word = 0;
    BCU(cudaMemcpyAsync(clocks, bt->d_clk, bt->nbox * sizeof(mhdgpu_clock), cudaMemcpyDeviceToHost, s),
        "mhdgpu_batch_read_clocks");
    BCU(cudaMemcpyAsync(&abort_word, bt->d_abort, sizeof(unsigned), cudaMemcpyDeviceToHost, s),
        "mhdgpu_batch_read_clocks");
    BCU(cudaStreamSynchronize(s), "mhdgpu_batch_read_clocks");
    if (abort_word) return bfail(MHD_ERR_TIMEOUT, "mhdgpu_batch: a dependency wait gave up; the state is invalid");
    for (int i = 0; i < bt->nbox; ++i)
        if (clocks[i].health & (MHD_HEALTH_NONFINITE | MHD_HEALTH_DENSITY))
            return bfail(MHD_ERR_UNPHYSICAL, "mhdgpu_batch: a box reports NaN/Inf or rho <= 0");
    return MHD_OK;
}

int mhdgpu_batch_set_schedule(mhdgpu_batch *bt, int axis, int threads, int ctas_per_sm)
{
    if (!bt) return bfail(MHD_ERR_ARG, "mhdgpu_batch_set_schedule: null handle");
    if (axis < 0 || axis > 2) return bfail(MHD_ERR_ARG, "mhdgpu_batch_set_schedule: axis must be 0, 1 or 2");
    if (threads != 64 && threads != 128 && threads != 256)
        return bfail(MHD_ERR_ARG, "mhdgpu_batch_set_schedule: threads must be 64, 128 or 256");
    if (ctas_per_sm < 1 || ctas_per_sm > 32)
        return bfail(MHD_ERR_ARG, "mhdgpu_batch_set_schedule: ctas_per_sm must be 1..32");
    const int old_t = bt->threads[axis], old_c = bt->cps[axis];
    bt->threads[axis] = threads;
    bt->cps[axis] = ctas_per_sm;
    bt->drop_parts();
    const int st = build_tables(*bt);
    if (st != MHD_OK) {
        bt->threads[axis] = old_t;
        bt->cps[axis] = old_c;
        build_tables(*bt);
    }
    return st;
}

int mhdgpu_batch_get_schedule(const mhdgpu_batch *bt, int axis, int *threads, int *ctas_per_sm)
{
    if (!bt || axis < 0 || axis > 2) return bfail(MHD_ERR_ARG, "mhdgpu_batch_get_schedule: bad argument");
    if (threads) *threads = bt->threads[axis];
    if (ctas_per_sm) *ctas_per_sm = bt->cps[axis];
    return MHD_OK;
}

// the batch's signature for the schedule cache: its boxes' sizes in order and
// the arithmetic policy of the calling thread (the class kernels differ by it)
static unsigned long long batch_signature(const mhdgpu_batch *bt)
{
    Fnv64 h;
    h.add(bt->nbox);
    for (const BoxDesc &d : bt->box) {
        h.add(d.nx);
        h.add(d.ny);
        h.add(d.nz);
    }
    h.add(math_mode());
    return h.h;
}

int mhdgpu_batch_schedule_save(const mhdgpu_batch *bt, const char *path)
{
    if (!bt || !path) return bfail(MHD_ERR_ARG, "mhdgpu_batch_schedule_save: null argument");
    FILE *f = fopen(path, "w");
    if (!f) return bfail(MHD_ERR_ARG, "mhdgpu_batch_schedule_save: cannot open the file");
    fprintf(f, "{\n  \"format\": \"mhdgpu batch schedule 1\",\n  \"device\": \"%s\",\n"
               "  \"signature\": \"%016llx\",\n  \"boxes\": %d,\n  \"schedule\": [",
            tune_device_name().c_str(), batch_signature(bt), bt->nbox);
    for (int a = 0; a < 3; ++a)
        fprintf(f, "%s\n    {\"axis\": %d, \"threads\": %d, \"ctas_per_sm\": %d}", a ? "," : "", a,
                bt->threads[a], bt->cps[a]);
    fprintf(f, "\n  ]\n}\n");
    if (fclose(f) != 0) return bfail(MHD_ERR_ARG, "mhdgpu_batch_schedule_save: write failed");
    return MHD_OK;
}

int mhdgpu_batch_schedule_load(mhdgpu_batch *bt, const char *path, int *applied)
{
    if (applied) *applied = 0;
    if (!bt || !path) return bfail(MHD_ERR_ARG, "mhdgpu_batch_schedule_load: null argument");
    std::string text, fmt, dev, sig;
    if (!read_text(path, text)) return bfail(MHD_ERR_ARG, "mhdgpu_batch_schedule_load: cannot read the file");
    if (!json_string(text, "format", fmt) || fmt != "mhdgpu batch schedule 1" || !json_string(text, "device", dev) ||
        !json_string(text, "signature", sig))
        return bfail(MHD_ERR_ARG, "mhdgpu_batch_schedule_load: not a batch schedule");
    char mine[32];
    snprintf(mine, sizeof mine, "%016llx", batch_signature(bt));
    if (!same_device(dev, tune_device_name()) || sig != mine) return MHD_OK;   // another device or batch
    int thr[3], cps[3], seen = 0;
    for (size_t p = text.find("{\"axis\""); p != std::string::npos && seen < 3; p = text.find("{\"axis\"", p + 1)) {
        int a, t, c;
        if (sscanf(text.c_str() + p, " { \"axis\" : %d , \"threads\" : %d , \"ctas_per_sm\" : %d }", &a, &t, &c) != 3 ||
            a != seen)
            return bfail(MHD_ERR_ARG, "mhdgpu_batch_schedule_load: malformed schedule");
        thr[a] = t;
        cps[a] = c;
        ++seen;
    }
    if (seen != 3) return bfail(MHD_ERR_ARG, "mhdgpu_batch_schedule_load: malformed schedule");
    for (int a = 0; a < 3; ++a) {
        const int st = mhdgpu_batch_set_schedule(bt, a, thr[a], cps[a]);
        if (st != MHD_OK) return st;
    }
    if (applied) *applied = 1;
    return MHD_OK;
}

int mhdgpu_batch_inject_stall(mhdgpu_batch *bt)
{
    if (!bt) return bfail(MHD_ERR_ARG, "mhdgpu_batch_inject_stall: null handle");
    bt->stall_extra = 1;
    return MHD_OK;
}

int mhdgpu_batch_tune(mhdgpu_batch *bt, mhdgpu_stream_t stream)
{
    if (!bt) return bfail(MHD_ERR_ARG, "mhdgpu_batch_tune: null handle");
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = bt->nbox;
    // snapshot of the state and the clocks
    long long cells = 0;
    for (const BoxDesc &d : bt->box) cells += (long long)d.nx * d.ny * d.nz;
    float *snap = nullptr;
    mhdgpu_clock *csnap = nullptr;
    BCU(cudaMalloc(&snap, 8 * sizeof(float) * (size_t)cells), "mhdgpu_batch_tune");
    if (cudaMalloc(&csnap, nb * sizeof(mhdgpu_clock)) != cudaSuccess) {
        cudaFree(snap);
        return bcuda(cudaErrorMemoryAllocation, "mhdgpu_batch_tune");
    }
    cudaEvent_t ev[7] = {};
    int st = MHD_OK;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 7 && e == cudaSuccess; ++i) e = cudaEventCreate(&ev[i]);
    long long off = 0;
    for (int i = 0; i < nb && e == cudaSuccess; ++i) {
        const BoxDesc &d = bt->box[i];
        const size_t nc = (size_t)d.nx * d.ny * d.nz;
        e = cudaMemcpyAsync(snap + 8 * off, d.u, 5 * nc * sizeof(float), cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(snap + 8 * off + 5 * nc, d.b, 3 * nc * sizeof(float), cudaMemcpyDeviceToDevice, s);
        off += nc;
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(csnap, bt->d_clk, nb * sizeof(mhdgpu_clock), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) st = bcuda(e, "mhdgpu_batch_tune");
    const int keep_t[3] = {bt->threads[0], bt->threads[1], bt->threads[2]};
    const int keep_c[3] = {bt->cps[0], bt->cps[1], bt->cps[2]};
    float best[3] = {1e30f, 1e30f, 1e30f};
    int best_t[3] = {keep_t[0], keep_t[1], keep_t[2]}, best_c[3] = {keep_c[0], keep_c[1], keep_c[2]};
    for (int ti = 0; ti < 3 && st == MHD_OK; ++ti) {
        for (int cps : {2, 4, 8}) {
            if (st != MHD_OK) break;
            for (int a = 0; a < 3; ++a) {
                bt->threads[a] = kThreadChoices[ti];
                bt->cps[a] = cps;
            }
            if (build_tables(*bt) != MHD_OK) continue;   // this schedule does not fit: skip it
            float tsum[3] = {0, 0, 0};
            for (int rep = 0; rep < 5 && st == MHD_OK; ++rep) {
                st = launch_step(*bt, s, ev, true);
                if (st != MHD_OK) break;
                if ((e = cudaEventSynchronize(ev[6])) != cudaSuccess) { st = bcuda(e, "mhdgpu_batch_tune"); break; }
                if (rep == 0) continue;   // warm-up
                for (int sw = 0; sw < 6; ++sw) {
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, ev[sw], ev[sw + 1]);
                    tsum[kSweepAxis[sw]] += ms;
                }
            }
            for (int a = 0; a < 3; ++a) {
                if (tsum[a] < best[a]) {
                    best[a] = tsum[a];
                    best_t[a] = kThreadChoices[ti];
                    best_c[a] = cps;
                }
            }
        }
    }
    for (int a = 0; a < 3; ++a) {
        bt->threads[a] = st == MHD_OK ? best_t[a] : keep_t[a];
        bt->cps[a] = st == MHD_OK ? best_c[a] : keep_c[a];
    }
    bt->drop_parts();
    const int st2 = build_tables(*bt);
    // restore the state, the clocks and the counters
    off = 0;
    e = cudaSuccess;
    for (int i = 0; i < nb && e == cudaSuccess; ++i) {
        const BoxDesc &d = bt->box[i];
        const size_t nc = (size_t)d.nx * d.ny * d.nz;
        e = cudaMemcpyAsync(d.u, snap + 8 * off, 5 * nc * sizeof(float), cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d.b, snap + 8 * off + 5 * nc, 3 * nc * sizeof(float), cudaMemcpyDeviceToDevice, s);
        off += nc;
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(bt->d_clk, csnap, nb * sizeof(mhdgpu_clock), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    for (int i = 0; i < 7; ++i)
        if (ev[i]) cudaEventDestroy(ev[i]);
    cudaFree(snap);
    cudaFree(csnap);
    if (st != MHD_OK) return st;
    if (e != cudaSuccess) return bcuda(e, "mhdgpu_batch_tune restore");
    return st2;
}

}  // extern "C"
