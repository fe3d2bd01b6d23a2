// gbp_batch.cpp -- host side of the batched MGPCG (BatchRunner).
//
// build(): uploads the level table, the per-scene table, the tails and the
// work lists of a plan. solve(): initial FP64 residual over every scene,
// then replays a CUDA graph of `chunk` iterations (one launch per kernel per
// iteration for the whole batch) and reads one counter -- the number of
// scenes not done -- between replays.
#include "gbp_batch.h"

#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>

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

int blocks_for(int items, int grid_blocks) { return std::max(1, std::min(items, grid_blocks)); }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); null if the driver does not provide it.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// A 3D FP32 tensor map over an nx x ny x nz array with the given box.
bool encode_map(CUtensorMap *m, const float *ptr, int nx, int ny, int nz, unsigned bx, unsigned by, unsigned bz) {
    auto enc = tensor_map_encoder();
    if (!enc || !ptr) return false;
    cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    cuuint64_t strides[2] = {(cuuint64_t)nx * 4, (cuuint64_t)nx * ny * 4};
    cuuint32_t box[3] = {bx, by, bz};
    cuuint32_t es[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(ptr), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The STAGE_MAPS maps of a fine FP32 level, or false if the level does not
// qualify: 3D, 4-plane tiles (one tile per item), nx a multiple of 8 (rows
// of the level and of its coarse grid are multiples of 16 bytes, every box
// x start a multiple of 4 floats), every array 16-byte aligned.
bool stage_maps(const BLevel<float> &L, const BScene<float> &S, CUtensorMap *m) {
    const Grid &g = L.g, &c = L.gc;
    if (g.dim != 3 || g.tz != ST_TZ || g.nx % 8 != 0 || !L.vec || c.nx % 4 != 0) return false;
    for (const void *p : {(const void *)L.b, (const void *)L.inv, (const void *)L.x, (const void *)L.cx,
                          (const void *)L.cy, (const void *)L.cz, (const void *)L.diag, (const void *)L.xc,
                          (const void *)S.p, (const void *)S.q})
        if (!p || (uintptr_t)p % 16 != 0) return false;
    const unsigned HX = ST_TX + 8, HY = ST_TY + 2, HZ = ST_TZ + 2;
    return encode_map(&m[SM_B_HALO], L.b, g.nx, g.ny, g.nz, HX, HY, HZ) &&
           encode_map(&m[SM_INV_HALO], L.inv, g.nx, g.ny, g.nz, HX, HY, HZ) &&
           encode_map(&m[SM_X_HALO], L.x, g.nx, g.ny, g.nz, HX, HY, HZ) &&
           encode_map(&m[SM_P_HALO], S.p, g.nx, g.ny, g.nz, HX, HY, HZ) &&
           encode_map(&m[SM_CX], L.cx, g.nx, g.ny, g.nz, HX, ST_TY, ST_TZ) &&
           encode_map(&m[SM_CY], L.cy, g.nx, g.ny, g.nz, ST_TX, ST_TY + 1, ST_TZ) &&
           encode_map(&m[SM_CZ], L.cz, g.nx, g.ny, g.nz, ST_TX, ST_TY, ST_TZ + 1) &&
           encode_map(&m[SM_B_OWN], L.b, g.nx, g.ny, g.nz, ST_TX, ST_TY, ST_TZ) &&
           encode_map(&m[SM_INV_OWN], L.inv, g.nx, g.ny, g.nz, ST_TX, ST_TY, ST_TZ) &&
           encode_map(&m[SM_DIAG_OWN], L.diag, g.nx, g.ny, g.nz, ST_TX, ST_TY, ST_TZ) &&
           encode_map(&m[SM_XC], L.xc, c.nx, c.ny, c.nz, 40, 6, 4);
}
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
    d_fine_staged_ = d_fine_plain_ = nullptr;
    n_fine_staged_ = s_fine_staged_ = n_fine_plain_ = s_fine_plain_ = 0;
    d_tmaps_ = nullptr;
    staged_scene_.clear();
    d_part_ = nullptr;
    d_counters_ = nullptr;
    bytes_ = 0;
}

template <class T> int BatchRunner::build(const BatchPlan<T> &plan, int grid_blocks, int staging, cudaStream_t stream) {
    release();
    stage_mask_ = 0;
    for (int &o : occ_) o = 0;
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
    tail_bytes_ = plan.tail_bytes;
    {
        int dev = 0, sms = 0;
        RUN_CUDA(cudaGetDevice(&dev));
        RUN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        grid_blocks_ = std::min(MAX_GRID, std::max(1, sms * BatchOcc<T>::blocks));
        (void)grid_blocks;
    }
    mixed_ = sizeof(T) == 4;
    sms_ = std::max(1, grid_blocks_ / BatchOcc<T>::blocks);
    // the gather-first column kernels (FP32 uniform tiles of 4 planes on
    // vector levels) are launched only for lists that hold such tiles
    fine_col_ = false;
    if (sizeof(T) == 4)
        for (int ref : plan.fine_ref)
            if (plan.levels[ref].g.tz == 4 && plan.levels[ref].vec && plan.levels[ref].tcp) fine_col_ = true;
    // staged fine levels: their tensor maps, in one device array
    std::vector<BLevel<T>> levels = plan.levels;
    std::vector<int> staged_at(levels.size(), -1);
    staged_scene_.assign(plan.nscenes, 0);
    if constexpr (sizeof(T) == 4) {
        if (staging) {
            std::vector<CUtensorMap> maps;
            for (int s = 0; s < plan.nscenes && s < (int)plan.fine_ref.size(); ++s) {
                const int ref = plan.fine_ref[s];
                CUtensorMap m[STAGE_MAPS];
                if (!stage_maps(levels[ref], plan.scenes[s], m)) continue;
                staged_at[ref] = (int)maps.size();
                staged_scene_[s] = 1;
                maps.insert(maps.end(), m, m + STAGE_MAPS);
            }
            if (!maps.empty()) {
                void *d;
                if ((rc = upload(maps.data(), maps.size() * sizeof(CUtensorMap), &d))) return rc;
                d_tmaps_ = static_cast<CUtensorMap *>(d);
                for (size_t r = 0; r < levels.size(); ++r)
                    if (staged_at[r] >= 0) levels[r].tmap = d_tmaps_ + staged_at[r];
                RUN_CUDA(b_staged_enable());
            }
        }
    }
    if ((rc = upload(levels.data(), levels.size() * sizeof(BLevel<T>), &d_levels_))) return rc;
    if ((rc = upload(plan.scenes.data(), plan.scenes.size() * sizeof(BScene<T>), &d_scenes_))) return rc;
    {
        void *d;
        if ((rc = upload(plan.scene_of.data(), plan.scene_of.size() * sizeof(int), &d))) return rc;
        d_scene_of_ = static_cast<int *>(d);
    }
    {
        // FP64 scratch of each scene's coarsest level, then the tail table
        void *d;
        const size_t per = 6 * (size_t)MG_COARSEST_MAX;
        if ((rc = upload(nullptr, sizeof(double) * per * std::max<size_t>(1, plan.tails.size()), &d))) return rc;
        std::vector<BTail<T>> tails = plan.tails;
        for (size_t s = 0; s < tails.size(); ++s) tails[s].c64 = static_cast<double *>(d) + s * per;
        if ((rc = upload(tails.data(), tails.size() * sizeof(BTail<T>), &d_tails_))) return rc;
    }
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
    // the fine list split into staged and plain segments (item positions
    // renumbered within each)
    {
        std::vector<BSeg> staged, plain;
        int ns = 0, np = 0;
        for (BSeg sg : plan.fine_pairs) {
            if (staged_at[sg.ref] >= 0) {
                sg.begin = ns;
                ns += sg.count;
                staged.push_back(sg);
            } else {
                sg.begin = np;
                np += sg.count;
                plain.push_back(sg);
            }
        }
        if ((rc = segs(staged, &d_fine_staged_, &s_fine_staged_))) return rc;
        if ((rc = segs(plain, &d_fine_plain_, &s_fine_plain_))) return rc;
        n_fine_staged_ = ns;
        n_fine_plain_ = np;
    }
    // coarse global levels 1..max_global-1: one cooperative launch per
    // V-cycle half, on at most as many blocks as stay resident
    coarse_ = CoarseLists{};
    coarse_blocks_ = 0;
    coarse_occ_ = 0;
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
    if (n_fine_staged_ > 0) stage_mask_ = (1 << STAGE_KINDS) - 1;
    // occupancy variants, tuned per precision and half-octave of fine cells
    long long cells = 0;
    for (const BScene<T> &sc : plan.scenes) cells += sc.g.ncell;
    const int bucket = cells > 0 ? (int)std::lround(2.0 * std::log2((double)cells)) : 0;
    const std::string key = std::string(sizeof(T) == 4 ? "f" : "d") + std::to_string(bucket) +
                            (stage_mask_ ? "s" : "") + "/" + std::to_string(plan.nscenes > 1 ? 2 : 1);
    if ((rc = tune_occupancy<T>(stream, key))) return rc;
    return GBP_OK;
}

template <class T> BLaunch BatchRunner::launch_for(int bk, int items, cudaStream_t st, int gate) const {
    const int occ = bk >= 0 ? occ_[bk] : 0;
    const int per_sm = occ ? occ : BatchOcc<T>::blocks;
    const bool col = fine_col_ && (bk == BK_PRESMOOTH || bk == BK_POST_BLACK || bk == BK_RED_DOT || bk == BK_SPMV);
    return BLaunch{blocks_for(items, std::min(MAX_GRID, sms_ * per_sm)), st, gate, d_scene_of_, d_counters_, occ,
                   col ? 1 : 0};
}

static MgSettings settings_of(const gbp_params &p) {
    MgSettings ms;
    ms.smooth = p.mg_smooth > 0 ? p.mg_smooth : 1;
    ms.coarsest_pairs = 4;
    ms.coarsest_pairs_warp = 8;
    ms.alpha = 1.6;
    return ms;
}

// The autotuner of occupancy: the fine-level kernels are compiled for 4, 5
// and 6 resident blocks of 256 threads per SM (more registers per thread, or
// more warps to hide latency); the best choice moves with the problem size
// (at 128^3 most run best with 4, at 256^3 red_dot and spmv with 6). For each
// tuned kernel this times the three variants on the batch's own work lists
// (one untimed launch each, then five rounds over the variants, the median
// of each variant's rounds, CUDA events on the solve's stream) and keeps the
// fastest. The launches run ungated on the scenes'
// arrays before the solve fills them: values do not change the work, every
// array they write is rewritten by the solve before it is read, and the
// solve resets the scalars and counters they touch. Choices are kept per
// precision and half-octave of the batch's fine cells. The same timing
// picks the grid of the cooperative coarse-level kernels (1, 2, 3 or 4 blocks
// per SM, or all that stay resident): fewer blocks make each grid-wide
// barrier cheaper, more hide the loads of the larger coarse levels.
template <class T> int BatchRunner::tune_occupancy(cudaStream_t st, const std::string &key) {
    static std::mutex mu;
    static std::map<std::string, std::vector<int>> cache;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = cache.find(key);
        if (it != cache.end()) {
            for (int k = 0; k < BK_TUNED; ++k) occ_[k] = it->second[k];
            // blocks per SM of the cooperative grid (0: all that stay resident)
            const int f = it->second[BK_TUNED];
            if (f > 0) coarse_blocks_ = std::min(coarse_blocks_, sms_ * f);
            coarse_occ_ = it->second[BK_TUNED + 1];
            return GBP_OK;
        }
    }
    if (max_global_ < 1) return GBP_OK;
    std::memset(h_counters_, 0, sizeof(BatchCounters));
    h_counters_->remaining = nscenes_;
    RUN_CUDA(cudaMemcpyAsync(d_counters_, h_counters_, sizeof(BatchCounters), cudaMemcpyHostToDevice, st));
    cudaEvent_t e0, e1;
    RUN_CUDA(cudaEventCreate(&e0));
    RUN_CUDA(cudaEventCreate(&e1));
    auto *lv = static_cast<const BLevel<T> *>(d_levels_);
    auto *sc = static_cast<const BScene<T> *>(d_scenes_);
    const gbp_params p{};
    cudaError_t err = cudaSuccess;
    auto pass = [&](int k) -> cudaError_t {
        switch (k) {
        case BK_PRESMOOTH: return fine_pass<T>(STAGE_PRESMOOTH, p, st, -1);
        case BK_RESTRICT:
            return b_restrict<T>(launch_for<T>(BK_RESTRICT, n_restrict_[0], st, -1), lv, d_restrict_[0],
                                 s_restrict_[0], n_restrict_[0], sc);
        case BK_POST_BLACK: return fine_pass<T>(STAGE_POST_BLACK, p, st, -1);
        case BK_RED_DOT: return fine_pass<T>(STAGE_RED_DOT, p, st, -1);
        case BK_DIRECTION:
            return b_direction<T>(launch_for<T>(BK_DIRECTION, n_fine_pairs_, st, -1), lv, d_fine_pairs_,
                                  s_fine_pairs_, n_fine_pairs_, sc);
        default: return fine_pass<T>(STAGE_SPMV, p, st, -1);
        }
    };
    // the variants are timed in turn, round after round, and each keeps the
    // median of its rounds: a drift of the clocks during the tuning (the
    // first solves after idle) then weighs on every variant alike
    constexpr int kVariants = 3, kRounds = 5;
    const int variants[kVariants] = {4, 5, 6};
    for (int k = 0; k < BK_TUNED && err == cudaSuccess; ++k) {
        float t[kVariants][kRounds] = {};
        for (int v = 0; v < kVariants && err == cudaSuccess; ++v) {
            occ_[k] = variants[v];
            err = pass(k);  // first launch of the variant, untimed
        }
        for (int r = 0; r < kRounds && err == cudaSuccess; ++r)
            for (int v = 0; v < kVariants && err == cudaSuccess; ++v) {
                occ_[k] = variants[v];
                err = cudaEventRecord(e0, st);
                if (err == cudaSuccess) err = pass(k);
                if (err == cudaSuccess) err = cudaEventRecord(e1, st);
                if (err == cudaSuccess) err = cudaEventSynchronize(e1);
                if (err == cudaSuccess) err = cudaEventElapsedTime(&t[v][r], e0, e1);
            }
        if (err != cudaSuccess) break;
        int pick = 0;
        float best = 0.f;
        for (int v = 0; v < kVariants; ++v) {
            std::sort(t[v], t[v] + kRounds);
            if (!pick || t[v][kRounds / 2] < best) {
                best = t[v][kRounds / 2];
                pick = variants[v];
            }
        }
        occ_[k] = pick;
    }
    int coarse_per_sm = 0;  // the cooperative grid's blocks per SM, 0: all resident (kept per key)
    if (err == cudaSuccess && coarse_blocks_ > 0) {
        const MgSettings ms = settings_of(p);
        const int full = coarse_blocks_;
        float best = 0.f;
        int pick = full;
        coarse_per_sm = 0;
        // (blocks per SM, register variant): 2 = launch bounds of 2 blocks
        // per SM (no spills), 0 = the precision's default bounds
        const int cand[6][2] = {{1, 2}, {2, 2}, {2, 0}, {3, 0}, {4, 0}, {0, 0}};
        coarse_occ_ = 0;
        std::vector<std::pair<int, int>> tried;
        for (const auto &cv : cand) {
            const int f = cv[0], occ = cv[1];
            const int nb = f ? std::min(full, sms_ * f) : full;
            if (occ == 2 && nb > 2 * sms_) continue;  // not all resident with that variant
            if (std::find(tried.begin(), tried.end(), std::make_pair(nb, occ)) != tried.end()) continue;
            tried.emplace_back(nb, occ);
            auto run = [&]() {
                cudaError_t e = b_coarse_descend<T>(BLaunch{nb, st, -1, d_scene_of_, d_counters_, occ}, lv, coarse_, sc, ms);
                if (e == cudaSuccess)
                    e = b_coarse_ascend<T>(BLaunch{nb, st, -1, d_scene_of_, d_counters_, occ}, lv, coarse_, sc, ms,
                                           T(ms.alpha));
                return e;
            };
            float t[3] = {0.f, 0.f, 0.f};
            err = run();
            for (int r = 0; r < 3 && err == cudaSuccess; ++r) {
                err = cudaEventRecord(e0, st);
                if (err == cudaSuccess) err = run();
                if (err == cudaSuccess) err = cudaEventRecord(e1, st);
                if (err == cudaSuccess) err = cudaEventSynchronize(e1);
                if (err == cudaSuccess) err = cudaEventElapsedTime(&t[r], e0, e1);
            }
            if (err != cudaSuccess) break;
            std::sort(t, t + 3);
            if (best == 0.f || t[1] < best) {
                best = t[1];
                pick = nb;
                coarse_per_sm = f;
                coarse_occ_ = occ;
            }
        }
        coarse_blocks_ = pick;
        if (err == cudaSuccess) {
            // a barrier that ran out of its wait is an error here as in a solve
            RUN_CUDA(cudaMemcpyAsync(h_counters_, d_counters_, sizeof(BatchCounters), cudaMemcpyDeviceToHost, st));
            RUN_CUDA(cudaStreamSynchronize(st));
            if (h_counters_->bar_err) err = cudaErrorLaunchTimeout;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess)
        return fail(GBP_ERR_CUDA, std::string("tuning kernel occupancy: ") + cudaGetErrorString(err));
    std::lock_guard<std::mutex> lock(mu);
    std::vector<int> choice(occ_, occ_ + BK_TUNED);
    choice.push_back(coarse_per_sm);
    choice.push_back(coarse_occ_);
    cache[key] = choice;
    return GBP_OK;
}

// One pass over the fine levels: the staged ones in one launch, the others
// with the direct-load kernel.
template <class T> cudaError_t BatchRunner::fine_pass(int kind, const gbp_params &p, cudaStream_t st, int gate) {
    const MgSettings ms = settings_of(p);
    auto *lv = static_cast<const BLevel<T> *>(d_levels_);
    auto *sc = static_cast<const BScene<T> *>(d_scenes_);
    cudaError_t e = cudaSuccess;
    // the plain pass covers every fine level unless this pass runs staged
    const BSeg *segs = d_fine_pairs_;
    int nseg = s_fine_pairs_, n = n_fine_pairs_;
    if constexpr (sizeof(T) == 4) {
        if (n_fine_staged_ > 0 && (stage_mask_ >> kind & 1)) {
            e = b_staged(kind, BLaunch{std::min(n_fine_staged_, sms_), st, gate, d_scene_of_, d_counters_}, lv,
                         d_fine_staged_, s_fine_staged_, n_fine_staged_, sc, d_part_, (float)ms.alpha);
            segs = d_fine_plain_;
            nseg = s_fine_plain_;
            n = n_fine_plain_;
        }
    }
    if (e != cudaSuccess || n == 0) return e;
    const int bk = kind == STAGE_PRESMOOTH ? BK_PRESMOOTH
                   : kind == STAGE_POST_BLACK ? BK_POST_BLACK
                   : kind == STAGE_RED_DOT ? BK_RED_DOT
                                           : BK_SPMV;
    const BLaunch L = launch_for<T>(bk, n, st, gate);
    switch (kind) {
    case STAGE_PRESMOOTH: return b_presmooth<T>(L, lv, segs, nseg, n, sc);
    case STAGE_POST_BLACK: return b_post_black<T>(L, lv, segs, nseg, n, sc, T(ms.alpha));
    case STAGE_RED_DOT: return b_red_dot<T>(L, lv, segs, nseg, n, sc, d_part_);
    default: return b_spmv<T>(L, lv, segs, nseg, n, sc, d_part_);
    }
}

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
        e = fine_pass<T>(STAGE_PRESMOOTH, p, st, gate);
        ++*nodes;
        for (int s = 1; s < ms.smooth && e == cudaSuccess; ++s) {
            e = b_sweep<T>(L(n_pair_[l]), lv, d_pair_[l], s_pair_[l], n_pair_[l], sc, 0);
            if (e == cudaSuccess) e = b_sweep<T>(L(n_pair_[l]), lv, d_pair_[l], s_pair_[l], n_pair_[l], sc, 1);
            *nodes += 2;
        }
        if (e == cudaSuccess)
            e = b_restrict<T>(launch_for<T>(BK_RESTRICT, n_restrict_[l], st, gate), lv, d_restrict_[l],
                              s_restrict_[l], n_restrict_[l], sc);
        ++*nodes;
    }
    if (e == cudaSuccess && max_global_ > 1) {
        e = b_coarse_descend<T>(BLaunch{coarse_blocks_, st, gate, d_scene_of_, d_counters_, coarse_occ_}, lv, coarse_, sc, ms);
        ++*nodes;
    }
    if (e == cudaSuccess && tail_bytes_ > 0) {
        e = b_tail<T>(BLaunch{nscenes_, st, gate, d_scene_of_, d_counters_}, tl, nscenes_, sc, ms);
        ++*nodes;
    }
    // ascend: the coarse global levels in one launch, then the fine level
    if (e == cudaSuccess && max_global_ > 1) {
        e = b_coarse_ascend<T>(BLaunch{coarse_blocks_, st, gate, d_scene_of_, d_counters_, coarse_occ_}, lv, coarse_, sc, ms,
                               T(ms.alpha));
        ++*nodes;
    }
    if (e == cudaSuccess && max_global_ > 0) {
        const int l = 0;
        e = fine_pass<T>(STAGE_POST_BLACK, p, st, gate);
        ++*nodes;
        for (int s = 1; s < ms.smooth && e == cudaSuccess; ++s) {
            e = b_sweep<T>(L(n_pair_[l]), lv, d_pair_[l], s_pair_[l], n_pair_[l], sc, 0);
            if (e == cudaSuccess) e = b_sweep<T>(L(n_pair_[l]), lv, d_pair_[l], s_pair_[l], n_pair_[l], sc, 1);
            *nodes += 2;
        }
        if (e == cudaSuccess) e = fine_pass<T>(STAGE_RED_DOT, p, st, gate);
        ++*nodes;
    }
    // CG on the fine level
    if (e == cudaSuccess)
        e = b_direction<T>(launch_for<T>(BK_DIRECTION, n_fine_pairs_, st, gate), lv, d_fine_pairs_, s_fine_pairs_,
                           n_fine_pairs_, sc);
    if (e == cudaSuccess) e = fine_pass<T>(STAGE_SPMV, p, st, gate);
    if (e == cudaSuccess)
        e = b_update<T>(L(n_fine_pairs_), lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc, d_part_, mixed_ ? 1 : 0, d_counters_);
    *nodes += 3;
    if (mixed_ && e == cudaSuccess) {
        const BLaunch L2{blocks_for(n_fine_pairs_, grid_blocks_), st, 2, d_scene_of_, d_counters_};
        // x64 += d, r64 -= A d and the outer stopping rule, in one pass
        e = b_refine_residual<T>(L2, lv, d_fine_pairs_, s_fine_pairs_, n_fine_pairs_, sc, d_part_, 0, p.residual,
                                 p.max_iterations, inner_rel_, kInnerMax, d_counters_);
        *nodes += 1;
    }
    return e;
}

template <class T> int BatchRunner::solve(const gbp_params &p, cudaStream_t st, long long *launches) {
    inner_rel_ = p.inner_tolerance > 0 ? p.inner_tolerance : 1e-3;
    auto *lv = static_cast<const BLevel<T> *>(d_levels_);
    auto *sc = static_cast<const BScene<T> *>(d_scenes_);
    std::memset(h_counters_, 0, sizeof(BatchCounters));
    h_counters_->remaining = nscenes_;
    h_counters_->test_what = test_what_;
    h_counters_->test_block = test_block_;
    h_counters_->test_polls = test_polls_;
    test_what_ = test_block_ = test_polls_ = 0;  // one solve only
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
            return fail(GBP_ERR_CUDA, h_counters_->bar_err == 2
                                          ? "staged fine-level kernels: a tile wait ran out (solve abandoned)"
                                          : "coarse-level kernels: a grid barrier wait ran out (solve abandoned)");
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
    case 0: launch = [&]() { return fine_pass<T>(STAGE_PRESMOOTH, gbp_params{}, st, 0); }; break;
    case 1:
        launch = [&]() {
            return b_restrict<T>(launch_for<T>(BK_RESTRICT, n_restrict_[0], st, 0), lv, d_restrict_[0],
                                 s_restrict_[0], n_restrict_[0], sc);
        };
        break;
    case 2:
        launch = [&]() { return fine_pass<T>(STAGE_POST_BLACK, gbp_params{}, st, 0); };
        break;
    case 3: launch = [&]() { return fine_pass<T>(STAGE_RED_DOT, gbp_params{}, st, 0); }; break;
    case 4:
        launch = [&]() {
            return b_direction<T>(launch_for<T>(BK_DIRECTION, n_fine_pairs_, st, 0), lv, d_fine_pairs_,
                                  s_fine_pairs_, n_fine_pairs_, sc);
        };
        break;
    case 5: launch = [&]() { return fine_pass<T>(STAGE_SPMV, gbp_params{}, st, 0); }; break;
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

template int BatchRunner::build<double>(const BatchPlan<double> &, int, int, cudaStream_t);
template int BatchRunner::build<float>(const BatchPlan<float> &, int, int, cudaStream_t);
template int BatchRunner::solve<double>(const gbp_params &, cudaStream_t, long long *);
template int BatchRunner::solve<float>(const gbp_params &, cudaStream_t, long long *);
template int BatchRunner::bench<double>(int, int, cudaStream_t, float *);
template int BatchRunner::bench<float>(int, int, cudaStream_t, float *);

}  // namespace gbp
