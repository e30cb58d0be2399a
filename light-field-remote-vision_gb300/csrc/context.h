// context.h -- the lfrv_ctx object: device, stream, launch counter and the device workspace.
#pragma once

#include "kernels.h"
#include "lfrv.h"
#include "lfrv_internal.h"

#include <cuda_runtime.h>

#include <atomic>
#include <map>
#include <string>
#include <vector>

namespace lfrv {

void check_cuda(cudaError_t e, const char *what);
#define LFRV_CUDA(call) ::lfrv::check_cuda((call), #call)

// Growable device allocation owned by a context.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    void ensure(size_t b);
    void release();
    template <class T> T *as() const { return static_cast<T *>(p); }
    ~DevBuf() { release(); }
};

// Device workspace of one solve. Buffers are grown on demand and kept between calls.
struct Workspace {
    // per view
    DevBuf img, tau, dp, wgt, res, vgrad, depth, tau_in, dpart_in, cams;
    // inverse footprint map
    DevBuf b_count, b_start, b_entries, b_aux, b_mask;
    // target
    DevBuf U, Ua, Ub, Uprev, P, Pa, F, G, g, g0, tmp, cov, norm, vis, Xq, gx, gy, mask, zkey, zbuf, zdefer;
    // gradient data term (dt_beta)
    DevBuf lapU, resg, ugrad;
    // target depth keys of the warps-from-depth path
    DevBuf ukey;
    // batched targets: per-job buffers and the launch descriptors
    DevBuf batch, batch_meta;
    // scratch state of the autotuner's trial launches
    DevBuf tune;
    // learned warm start: network input (NHWC BF16) and the seeded CG iterate
    DevBuf learn_in, seed;
    // CG
    DevBuf r, d, q, U0, holes, hole_count;
    // reductions and persistent-solver state; per-iteration energies of the current call (energy trace)
    DevBuf partial, sums, state, barrier, trace;
    // push-pull pyramid
    DevBuf pp_img, pp_vis, pp_tmp, pp_orig;
    // host staging for the host-buffer entry points
    DevBuf in_views, in_tau, in_dpart, in_init, out_img;
    // host-buffer batched calls: one device copy per distinct light field (views, depth) and the outputs
    DevBuf hb_in, hb_out;
    // batched calls: the view gradients of each distinct light field, shared by the jobs that render from it
    DevBuf vg_pool;
    // corrected IBR_color: iterates, data gradients and metric (15 N floats), the FP64 dual / momentum fields (24 N)
    DevBuf tv;
    // the device scene generator's planes and bumps
    DevBuf scene;
    // the device-side loop state of a graph-driven corrected IBR_color solve
    DevBuf tvloop;
};

// Per-kernel CUDA-event timing: a fixed pool of event pairs recorded in-stream. When the pool is full the
// stream is synchronised and the recorded pairs are folded into per-name totals (profiling mode only).
struct KernelProfiler {
    struct Rec {
        const char *name;
        int slot;
    };
    std::vector<cudaEvent_t> ev;  // 2 per slot
    std::vector<Rec> recs;
    int next = 0;
    std::vector<std::string> names;  // totals in first-seen order
    std::vector<double> ms;
    std::vector<long long> count;
    void init(int slots);
    void destroy();
    void reset();
    void fold();  // waits for the recorded pairs (on any stream), adds them to the totals, frees the pool
    int begin(const char *name, cudaStream_t st);
    void end(int slot, cudaStream_t st);
};

// Statistics left on the device by persistent solvers of the current call, read after the stream completes.
struct Pending {
    bool cg = false, hole_fill = false;
    bool barrier = false;  // a persistent kernel used the grid barrier since the last check (error word armed)
    lfrv_stats *stats = nullptr;
    double gap_tol = 0.0;
    // energy trace requested by the caller: entries kept in ws.trace on the device, copied to trace_host once the
    // stream has completed. trace_len >= 0 is the entry count known on the host; -1 takes the CG's iteration
    // count from the device state
    double *trace_host = nullptr;
    int trace_cap = 0;
    int trace_len = -1;
};

// Bumped by every workspace allocation and release: a captured graph holds workspace pointers and is replayed
// only while the epoch it was captured at is current.
extern std::atomic<unsigned long long> g_alloc_epoch;

// One captured render call (lfrv_render_view_dev): the call's argument bytes, and once the same call has run
// uncaptured, its executable graph with the host-side state the capture left (pending statistics, launches).
struct RenderGraph {
    std::vector<unsigned char> key;
    bool seen = false;     // this key ran once uncaptured (its workspace is allocated)
    bool failed = false;   // capturing this key failed: it runs uncaptured
    cudaGraphExec_t exec = nullptr;
    unsigned long long epoch = 0;
    Pending pending;
    long long launches = 0;
    void reset(std::vector<unsigned char> k) {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        key = std::move(k);
        seen = false;
        failed = false;
    }
};

}  // namespace lfrv

struct lfrv_ctx {
    // host-buffer calls upload on a second stream so the copies overlap the warp stage (created on first use)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t up_start = nullptr, up_depth[4] = {}, up_views = nullptr;
    cudaEvent_t out_ready = nullptr;  // a batched host-buffer call's job output is final (its download may start)
    // work that depends only on a call's inputs runs on a side stream, joined by event (created on first use)
    cudaStream_t side_stream = nullptr;
    cudaEvent_t side_fork = nullptr, side_join = nullptr;
    lfrv::Pending pending;
    std::map<long long, int> rof_tuned;  // autotuned persistent-ROF variant per image size (W << 32 | H)
    std::map<long long, int> fgp_tuned;  // autotuned FGP variant per image size and arithmetic
    lfrv::KernelProfiler prof;
    bool profiling = false;
    int device = 0;
    cudaStream_t stream = nullptr;
    lfrv::LaunchCounter launches;
    lfrv::Workspace ws;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t vg_ready = nullptr;  // a batched call's shared view gradients are written
    lfrv::RenderGraph graph;  // replay of a repeated lfrv_render_view_dev call
    // the warp stage counted the inverse map's buckets for this geometry (W, H, dsf, V, n): the next bucket build
    // of the same geometry skips its count pass
    bool buckets_counted = false;
    long long counted_geometry[5] = {};
    const float *counted_tau = nullptr;  // the tau2 the counts were taken from
    // helper contexts (own stream and workspace) that prepare batched targets concurrently; created on first use
    std::vector<lfrv_ctx *> lanes;
    std::vector<cudaEvent_t> lane_done;
    bool owns_stream = false;
    bool lane = false;  // a helper context of a batched call (its stream already runs beside the others)
    double *host_sums = nullptr;  // pinned host copy of reduction sums (corrected IBR_color's stop test)
    // contexts of the corrected IBR_color jobs of a batched call (one per job, own stream and workspace)
    std::vector<lfrv_ctx *> tv_jobs;
};
