// gbp_batch.cpp -- host side of the batched MGPCG (BatchRunner).
//
// build(): uploads the level table, the per-scene table, the tails and the
// work lists of a plan. solve(): initial FP64 residual over every scene,
// then replays a CUDA graph of `chunk` iterations (one launch per kernel per
// iteration for the whole batch) and reads one counter -- the number of
// scenes not done -- between replays.
#include "gbp_batch.h"

#include <algorithm>
#include <cstring>
#include <functional>

namespace gbp {

namespace {
#define RUN_CUDA(call)                                                                                 \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return fail(e_ == cudaErrorMemoryAllocation ? GBP_ERR_OUT_OF_MEMORY : GBP_ERR_CUDA,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                          \
    } while (0)

constexpr int kChunk = 4;
constexpr int kInnerMax = 50;
}  // namespace

void BatchRunner::release() {
    if (graph_) {
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
    }
    graph_key_ = -1;
    for (void *p : owned_) cudaFree(p);
    owned_.clear();
    if (h_counters_) cudaFreeHost(h_counters_);
    h_counters_ = nullptr;
    d_levels_ = d_scenes_ = d_tails_ = nullptr;
    d_scene_of_ = nullptr;
    d_pair_.clear();
    d_restrict_.clear();
    n_pair_.clear();
    n_restrict_.clear();
    s_pair_.clear();
    s_restrict_.clear();
    d_fine_pairs_ = nullptr;
    d_part_ = nullptr;
    d_counters_ = nullptr;
    bytes_ = 0;
}

template <class T> int BatchRunner::build(const BatchPlan<T> &plan, int grid_blocks) {
    release();
    auto upload = [&](const void *src, size_t bytes, void **dst) -> int {
        void *d = nullptr;
        RUN_CUDA(cudaMalloc(&d, bytes ? bytes : 16));
        owned_.push_back(d);
        bytes_ += bytes;
        if (bytes && src) RUN_CUDA(cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice));
        else if (bytes) RUN_CUDA(cudaMemset(d, 0, bytes));
        *dst = d;
        return GBP_OK;
    };
    int rc;
    nscenes_ = plan.nscenes;
    max_global_ = plan.max_global;
    tail_smem_ = plan.tail_smem;
    {
        int dev = 0, sms = 0;
        RUN_CUDA(cudaGetDevice(&dev));
        RUN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        grid_blocks_ = std::min(MAX_GRID, std::max(1, sms * BatchOcc<T>::blocks));
        (void)grid_blocks;
    }
    mixed_ = sizeof(T) == 4;
    if ((rc = upload(plan.levels.data(), plan.levels.size() * sizeof(BLevel<T>), &d_levels_))) return rc;
    if ((rc = upload(plan.scenes.data(), plan.scenes.size() * sizeof(BScene<T>), &d_scenes_))) return rc;
    {
        void *d;
        if ((rc = upload(plan.scene_of.data(), plan.scene_of.size() * sizeof(int), &d))) return rc;
        d_scene_of_ = static_cast<int *>(d);
    }
    if ((rc = upload(plan.tails.data(), plan.tails.size() * sizeof(BTail<T>), &d_tails_))) return rc;
    size_t max_items = (size_t)plan.n_fine_pairs;
    auto segs = [&](const std::vector<BSeg> &list, BSeg **dst, int *nseg) -> int {
        void *d;
        int rc2 = upload(list.data(), list.size() * sizeof(BSeg), &d);
        *dst = static_cast<BSeg *>(d);
        *nseg = (int)list.size();
        return rc2;
    };
    d_pair_.assign(plan.max_global, nullptr);
    d_restrict_.assign(plan.max_global, nullptr);
    s_pair_.assign(plan.max_global, 0);
    s_restrict_.assign(plan.max_global, 0);
    n_pair_.assign(plan.n_pair.begin(), plan.n_pair.begin() + plan.max_global);
    n_restrict_.assign(plan.n_restrict.begin(), plan.n_restrict.begin() + plan.max_global);
    for (int l = 0; l < plan.max_global; ++l) {
        if ((rc = segs(plan.pair[l], &d_pair_[l], &s_pair_[l]))) return rc;
        if ((rc = segs(plan.restrict_[l], &d_restrict_[l], &s_restrict_[l]))) return rc;
        max_items = std::max(max_items, (size_t)plan.n_pair[l]);
    }
    if ((rc = segs(plan.fine_pairs, &d_fine_pairs_, &s_fine_pairs_))) return rc;
    n_fine_pairs_ = plan.n_fine_pairs;
    // coarse global levels 1..max_global-1: one cooperative launch per
    // V-cycle half, on at most as many blocks as stay resident
    coarse_ = CoarseLists{};
    coarse_blocks_ = 0;
    if (plan.max_global > 1) {
        coarse_.first = 1;
        coarse_.last = plan.max_global - 1;
        int most = 1;
        for (int l = 1; l < plan.max_global; ++l) {
            coarse_.pair[l] = d_pair_[l];
            coarse_.pair_seg[l] = s_pair_[l];
            coarse_.pair_n[l] = n_pair_[l];
            coarse_.restr[l] = d_restrict_[l];
            coarse_.restr_seg[l] = s_restrict_[l];
            coarse_.restr_n[l] = n_restrict_[l];
            most = std::max(most, std::max(n_pair_[l], n_restrict_[l]));
        }
        int dev = 0, sms = 0;
        RUN_CUDA(cudaGetDevice(&dev));
        RUN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int cap = b_coarse_capacity<T>(sms);
        if (cap < 1) return fail(GBP_ERR_CUDA, "coarse-level kernels: no resident block");
        coarse_blocks_ = std::min(cap, most);
    }
    void *d;
    max_items_ = (int)max_items;
    // two partials per item (the refinement keeps a max and a sum)
    if ((rc = upload(nullptr, sizeof(double) * 2 * (max_items + 1), &d))) return rc;
    d_part_ = static_cast<double *>(d);
    if ((rc = upload(nullptr, sizeof(BatchCounters), &d))) return rc;
    d_counters_ = static_cast<BatchCounters *>(d);
    RUN_CUDA(cudaMallocHost(&h_counters_, sizeof(BatchCounters)));
    if (tail_smem_ > 0) RUN_CUDA(b_tail_enable<T>(tail_smem_));
    return GBP_OK;
}

static MgSettings settings_of(const gbp_params &p) {
    MgSettings ms;
    ms.smooth = p.mg_smooth > 0 ? p.mg_smooth : 1;
    ms.coarsest_pairs = 4;
    ms.alpha = 1.6;
    return ms;
}

static int blocks_for(int items, int grid_blocks) { return std::max(1, std::min(items, grid_blocks)); }

template <class T> cudaError_t BatchRunner::enqueue_iteration(const gbp_params &p, cudaStream_t st, long long *nodes) {
    const int gate = mixed_ ? 1 : 0;
    const MgSettings ms = settings_of(p);
    auto *lv = static_cast<const BLevel<T> *>(d_levels_);
    auto *sc = static_cast<const BScene<T> *>(d_scenes_);
    auto *tl = static_cast<const BTail<T> *>(d_tails_);
    cudaError_t e = cudaSuccess;
    auto L = [&](int items) { return BLaunch{blocks_for(items, grid_blocks_), st, gate, d_scene_of_, d_counters_}; };
    // descend: the fine level, then the coarse global levels in one launch
    if (max_global_ > 0) {
        const int l = 0;
        e = b_presmooth<T>(L(n_pair_[l]), lv, d_pair_[l], s_pair_[l], n_pair_[l], sc);
        ++*nodes;
        for (int s = 1; s < ms.smooth && e == cudaSuccess; ++s) {
            e = b_sweep<T>(L(n_pair_[l]), lv, d_pair_[l], s_pair_[l], n_pair_[l], sc, 0);
            if (e == cudaSuccess) e = b_sweep<T>(L(n_pair_[l]), lv, d_pair_[l], s_pair_[l], n_pair_[l], sc, 1);
            *nodes += 2;
        }
        if (e == cudaSuccess) e = b_restrict<T>(L(n_restrict_[l]), lv, d_restrict_[l], s_restrict_[l], n_restrict_[l], sc);
        ++*nodes;
    }
    if (e == cudaSuccess && max_global_ > 1) {
        e = b_coarse_descend<T>(BLaunch{coarse_blocks_, st, gate, d_scene_of_, d_counters_}, lv, coarse_, sc, ms);
        ++*nodes;
    }
    if (e == cudaSuccess && tail_smem_ > 0) {
        e = b_tail<T>(BLaunch{nscenes_, st, gate, d_scene_of_, d_counters_}, tl, nscenes_, sc, ms, tail_smem_);
        ++*nodes;
    }
    // ascend: the coarse global levels in one launch, then the fine level
    if (e == cudaSuccess && max_global_ > 1) {
        e = b_coarse_ascend<T>(BLaunch{coarse_blocks_, st, gate, d_scene_of_, d_counters_}, lv, coarse_, sc, ms,
                               T(ms.alpha));
        ++*nodes;
    }
    if (e == cudaSuccess && max_global_ > 0) {
        const int l = 0;
        e = b_post_black<T>(L(n_pair_[l]), lv, d_pair_[l], s_pair_[l], n_pair_[l], sc, T(ms.alpha));
        ++*nodes;
        for (int s = 1; s < ms.smooth && e == cudaSuccess; ++s) {
            e = b_sweep<T>(L(n_pair_[l]), lv, d_pair_[l], s_pair_[l], n_pair_[l], sc, 0);
            if (e == cudaSuccess) e = b_sweep<T>(L(n_pair_[l]), lv, d_pair_[l], s_pair_[l], n_pair_[l], sc, 1);
            *nodes += 2;
        }
        if (e == cudaSuccess) e = b_red_dot<T>(L(n_fine_pairs_), lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc, d_part_);
        ++*nodes;
    }
    // CG on the fine level
    if (e == cudaSuccess) e = b_direction<T>(L(n_fine_pairs_), lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc);
    if (e == cudaSuccess) e = b_spmv<T>(L(n_fine_pairs_), lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc, d_part_);
    if (e == cudaSuccess)
        e = b_update<T>(L(n_fine_pairs_), lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc, d_part_, mixed_ ? 1 : 0, d_counters_);
    *nodes += 3;
    if (mixed_ && e == cudaSuccess) {
        const BLaunch L2{blocks_for(n_fine_pairs_, grid_blocks_), st, 2, d_scene_of_, d_counters_};
        e = b_refine_accumulate<T>(L2, lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc);
        if (e == cudaSuccess)
            e = b_refine_residual<T>(L2, lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc, d_part_, 0, p.residual,
                                     p.max_iterations, inner_rel_, kInnerMax, d_counters_);
        *nodes += 2;
    }
    return e;
}

template <class T> int BatchRunner::solve(const gbp_params &p, cudaStream_t st, long long *launches) {
    inner_rel_ = p.inner_tolerance > 0 ? p.inner_tolerance : 1e-3;
    auto *lv = static_cast<const BLevel<T> *>(d_levels_);
    auto *sc = static_cast<const BScene<T> *>(d_scenes_);
    std::memset(h_counters_, 0, sizeof(BatchCounters));
    h_counters_->remaining = nscenes_;
    RUN_CUDA(cudaMemcpyAsync(d_counters_, h_counters_, sizeof(BatchCounters), cudaMemcpyHostToDevice, st));
    // initial residual of every scene (also zeroes x64, sets thresholds)
    RUN_CUDA(b_refine_residual<T>(BLaunch{blocks_for(n_fine_pairs_, grid_blocks_), st, 0, d_scene_of_, d_counters_}, lv,
                                  d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc, d_part_, 1, p.residual, p.max_iterations, inner_rel_, kInnerMax,
                                  d_counters_));
    *launches += 1;
    const long long key = ((long long)(p.mg_smooth > 0 ? p.mg_smooth : 1) << 40) ^
                          (long long)(p.residual * 1e15) ^ ((long long)p.max_iterations << 8) ^
                          (long long)(inner_rel_ * 1e12);
    if (!graph_ || graph_key_ != key) {
        if (graph_) cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
        cudaGraph_t graph;
        long long nodes = 0;
        RUN_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        for (int it = 0; it < kChunk && e == cudaSuccess; ++it) e = enqueue_iteration<T>(p, st, &nodes);
        cudaError_t e2 = cudaStreamEndCapture(st, &graph);
        if (e != cudaSuccess || e2 != cudaSuccess)
            return fail(GBP_ERR_CUDA, std::string("capturing batched MGPCG iterations: ") +
                                          cudaGetErrorString(e != cudaSuccess ? e : e2));
        e = cudaGraphInstantiate(&graph_, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(GBP_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        graph_key_ = key;
        graph_nodes_ = nodes;
    }
    const long long max_chunks = (long long)p.max_iterations / kChunk + 64;
    for (long long k = 0; k < max_chunks; ++k) {
        RUN_CUDA(cudaMemcpyAsync(h_counters_, d_counters_, sizeof(BatchCounters), cudaMemcpyDeviceToHost, st));
        RUN_CUDA(cudaStreamSynchronize(st));
        if (h_counters_->bar_err)
            return fail(GBP_ERR_CUDA, "coarse-level kernels: a grid barrier wait ran out (solve abandoned)");
        if (h_counters_->remaining <= 0) return GBP_OK;
        RUN_CUDA(cudaGraphLaunch(graph_, st));
        *launches += graph_nodes_;
    }
    RUN_CUDA(cudaStreamSynchronize(st));
    return GBP_OK;
}

template <class T> int BatchRunner::bench(int which, int reps, cudaStream_t st, float *ms) {
    auto *lv = static_cast<const BLevel<T> *>(d_levels_);
    auto *sc = static_cast<const BScene<T> *>(d_scenes_);
    const MgSettings mset = settings_of(gbp_params{});
    std::function<cudaError_t()> launch;
    auto L = [&](int items) { return BLaunch{blocks_for(items, grid_blocks_), st, 0, d_scene_of_, d_counters_}; };
    switch (which) {
    case 0: launch = [&]() { return b_presmooth<T>(L(n_pair_[0]), lv, d_pair_[0], s_pair_[0], n_pair_[0], sc); }; break;
    case 1: launch = [&]() { return b_restrict<T>(L(n_restrict_[0]), lv, d_restrict_[0], s_restrict_[0], n_restrict_[0], sc); }; break;
    case 2:
        launch = [&]() { return b_post_black<T>(L(n_pair_[0]), lv, d_pair_[0], s_pair_[0], n_pair_[0], sc, T(mset.alpha)); };
        break;
    case 3: launch = [&]() { return b_red_dot<T>(L(n_fine_pairs_), lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc, d_part_); }; break;
    case 4: launch = [&]() { return b_direction<T>(L(n_fine_pairs_), lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc); }; break;
    case 5: launch = [&]() { return b_spmv<T>(L(n_fine_pairs_), lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc, d_part_); }; break;
    case 6:
        launch = [&]() {
            return b_update<T>(L(n_fine_pairs_), lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc, d_part_, 0, d_counters_);
        };
        break;
    default: return fail(GBP_ERR_INVALID_ARGUMENT, "bench: unknown kernel");
    }
    if (max_global_ < 1) return fail(GBP_ERR_INVALID_ARGUMENT, "bench: no multigrid level");
    // a live batch, so that no launch takes the idle exit
    std::memset(h_counters_, 0, sizeof(BatchCounters));
    h_counters_->remaining = nscenes_;
    RUN_CUDA(cudaMemcpyAsync(d_counters_, h_counters_, sizeof(BatchCounters), cudaMemcpyHostToDevice, st));
    cudaEvent_t e0, e1;
    RUN_CUDA(cudaEventCreate(&e0));
    RUN_CUDA(cudaEventCreate(&e1));
    RUN_CUDA(launch());
    RUN_CUDA(cudaEventRecord(e0, st));
    for (int i = 0; i < reps; ++i) RUN_CUDA(launch());
    RUN_CUDA(cudaEventRecord(e1, st));
    RUN_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / (reps > 0 ? reps : 1);
    return GBP_OK;
}

template int BatchRunner::build<double>(const BatchPlan<double> &, int);
template int BatchRunner::build<float>(const BatchPlan<float> &, int);
template int BatchRunner::solve<double>(const gbp_params &, cudaStream_t, long long *);
template int BatchRunner::solve<float>(const gbp_params &, cudaStream_t, long long *);
template int BatchRunner::bench<double>(int, int, cudaStream_t, float *);
template int BatchRunner::bench<float>(int, int, cudaStream_t, float *);

}  // namespace gbp
