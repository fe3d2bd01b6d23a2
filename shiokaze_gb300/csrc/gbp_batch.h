// gbp_batch.h -- batched MGPCG: one launch per kernel for many scenes.
//
// Every kernel of the multigrid-preconditioned CG iteration walks a work
// list of items; an item is one tile of one level of one scene. A launch
// therefore serves all scenes of a batch (of uneven sizes and depths) at
// once, and a CUDA graph of a few iterations serves the whole batch.
//
// Reductions are per scene and deterministic: each item writes its tile's
// partial, takes a ticket from its scene's counter, and the item that takes
// the scene's last ticket sums that scene's partials in item order. A
// scene's result therefore does not depend on which other scenes share the
// batch (the serving test checks this), and a single-scene solve is a batch
// of one.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gbp.h"
#include "gbp_internal.cuh"
#include "gbp_kernels.h"
#include "gbp_mg.h"

namespace gbp {

// One level of one scene as the batched kernels see it.
template <class T> struct BLevel {
    Grid g;
    const T *diag, *inv, *cx, *cy, *cz;  // cz == cy in 2D
    T *b, *x;
    const T *xc;  // x of the next coarser level (post-smoothing)
    T *bc;        // b of the next coarser level (restriction)
    Grid gc;      // the next coarser grid
    int scene;
    // pairs of this level (and, on level 0, of the scene's vectors) move as
    // 2-wide accesses: nx even and every such array 2-element aligned
    int vec;
};

// Per-scene state of the fine level.
template <class T> struct BScene {
    Grid g;
    T *x, *r, *z, *p, *q;  // PCG vectors (x: the correction in FP64 mode, d in mixed mode)
    // FP64 operator and refinement state
    Operator<double> A;
    const double *b, *prev;
    double *x64, *r64;
    Scalars *sc;
    int levels;  // multigrid levels of the scene
    int tail;    // first level of its shared-memory tail (== levels: none)
};

struct BItem {
    int ref;     // level table index
    int tile;    // first tile (in the kernel's tiling of that level)
    int ntiles;  // consecutive tiles of the item
    int begin;   // first item of this scene in the list
    int count;   // items of this scene in the list
};

// Resident blocks of BLOCK_THREADS per SM that the batched kernels of type
// T are compiled for (their launch bounds) and launched with (grid = SMs x
// this). The FP32 kernels move pairs of cells and want registers (48 a
// thread at 5 blocks); the FP64 kernels are bound by the FP64 pipe and want
// warps to hide its latency.
template <class T> struct BatchOcc;
template <> struct BatchOcc<float> {
    static constexpr int blocks = 5;
};
template <> struct BatchOcc<double> {
    static constexpr int blocks = 4;
};

// Tiles per item (items are the unit of load balance; reductions are per
// block, so small items cost little).
constexpr int BITEM_CELLS = 512;

// A work list is the concatenation of one segment per scene: items
// [begin, begin+count) of the list are tiles [k*m, k*m+m) of level `ref`.
// Kernels derive each item from its index, with no per-item load.
struct BSeg {
    int ref;
    int begin;
    int count;
    int m;       // tiles per item
    int ntiles;  // tiles of the level in this tiling
};

// Item w of a segment list; `seg` is the caller's cursor (items are visited
// in increasing order, so it only moves forward).
__host__ __device__ inline BItem item_at(const BSeg *segs, int nseg, int w, int &seg) {
    while (seg + 1 < nseg && w >= segs[seg + 1].begin) ++seg;
    const BSeg &s = segs[seg];
    const int k = w - s.begin;
    const int t = k * s.m;
    const int nt = s.ntiles - t < s.m ? s.ntiles - t : s.m;
    return BItem{s.ref, t, nt, s.begin, s.count};
}

template <class T> struct BTail {
    int nt;
    MgLevel<T> lv[MG_MAX_LEVELS];
};

// Tilings: pair tiles (64 x 8 x tz) for the red-black kernels, cell tiles
// (32 x 8 x tz) for the rest.
inline long long pair_tiles(const Grid &g) { return (long long)((g.nx + 63) / 64) * g.nty * g.ntz; }
inline long long cell_tiles(const Grid &g) { return g.ntiles; }

struct BatchCounters {
    int remaining;        // scenes not done
    int refine;           // scenes whose inner solve ended, awaiting refinement
    unsigned bar_count;   // grid barrier of the coarse-level kernels: arrivals
    unsigned bar_gen;     // ... and generation
    int bar_err;          // a barrier wait ran out (the solve is abandoned)
    int pad[3];
};

// Work lists of the global coarse levels [first, last] (first >= 1), run by
// one cooperative launch per V-cycle half.
struct CoarseLists {
    int first, last;
    const BSeg *pair[MG_MAX_LEVELS];
    int pair_seg[MG_MAX_LEVELS], pair_n[MG_MAX_LEVELS];
    const BSeg *restr[MG_MAX_LEVELS];
    int restr_seg[MG_MAX_LEVELS], restr_n[MG_MAX_LEVELS];
};

// Device tables and work lists of one batch, built on the host.
template <class T> struct BatchPlan {
    int nscenes = 0;
    int max_global = 0;                  // max over scenes of the tail level
    std::vector<BLevel<T>> levels;       // all scenes' global levels
    std::vector<int> scene_of;           // scene of each level entry
    std::vector<BScene<T>> scenes;
    std::vector<BTail<T>> tails;
    size_t tail_smem = 0;
    // work lists as segments: pair[l] (pair tiles of level l), restrict[l]
    // (cell tiles of level l+1), fine (pair tiles of level 0), with their
    // item counts
    std::vector<std::vector<BSeg>> pair, restrict_;
    std::vector<BSeg> fine_pairs;
    std::vector<int> n_pair, n_restrict;
    int n_fine_pairs = 0;
};

class BatchRunner {
public:
    BatchRunner() = default;
    ~BatchRunner() { release(); }
    BatchRunner(const BatchRunner &) = delete;
    BatchRunner &operator=(const BatchRunner &) = delete;

    // Uploads the plan (tables, lists) and sizes the partials. T = double
    // for the FP64 path, float for the inner solve of the mixed path.
    template <class T> int build(const BatchPlan<T> &plan, int grid_blocks);
    // Runs the solve after every scene's operator and hierarchy are set up:
    // initial residual, then graph replays until every scene is done.
    template <class T> int solve(const gbp_params &p, cudaStream_t stream, long long *launches);
    // Times reps launches of one kernel of the iteration (benchmarking):
    // 0 presmooth, 1 restrict, 2 post_black, 3 red_dot (fine level),
    // 4 direction, 5 spmv, 6 update.
    template <class T> int bench(int which, int reps, cudaStream_t stream, float *ms);
    void release();
    const char *error() const { return err_.c_str(); }
    size_t device_bytes() const { return bytes_; }

private:
    int fail(int code, const std::string &m) {
        err_ = m;
        return code;
    }
    template <class T> cudaError_t enqueue_iteration(const gbp_params &p, cudaStream_t stream, long long *nodes);
    std::string err_;
    bool mixed_ = false;
    int grid_blocks_ = 0;
    int nscenes_ = 0;
    int max_global_ = 0;
    size_t tail_smem_ = 0;
    size_t bytes_ = 0;
    std::vector<void *> owned_;
    // device copies
    void *d_levels_ = nullptr, *d_scenes_ = nullptr, *d_tails_ = nullptr;
    int *d_scene_of_ = nullptr;
    std::vector<BSeg *> d_pair_, d_restrict_;
    std::vector<int> n_pair_, n_restrict_, s_pair_, s_restrict_;  // items, segments
    BSeg *d_fine_pairs_ = nullptr;
    int n_fine_pairs_ = 0, s_fine_pairs_ = 0;
    double *d_part_ = nullptr;  // 3 x max items
    int max_items_ = 0;
    BatchCounters *d_counters_ = nullptr, *h_counters_ = nullptr;
    CoarseLists coarse_{};
    int coarse_blocks_ = 0;
    cudaGraphExec_t graph_ = nullptr;
    long long graph_key_ = -1;
    long long graph_nodes_ = 0;
    double inner_rel_ = 1e-3;
};

// Launch functions (batch_kernels.cu). `levels`, `scenes`, `items` are
// device arrays.
struct BLaunch {
    int blocks;
    cudaStream_t stream;
    int gate;
    const int *scene_of;  // scene of each level-table entry (reductions)
    BatchCounters *cnt;   // batch counters (idle and refinement checks)
};

template <class T>
cudaError_t b_presmooth(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n, const BScene<T> *scenes);
template <class T>
cudaError_t b_sweep(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n, const BScene<T> *scenes,
                    int color);
template <class T>
cudaError_t b_restrict(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                       const BScene<T> *scenes);
template <class T>
cudaError_t b_post_black(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                         const BScene<T> *scenes, T alpha);
template <class T>
cudaError_t b_red_dot(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n, const BScene<T> *scenes,
                      double *part);
template <class T>
cudaError_t b_tail(const BLaunch &L, const BTail<T> *tails, int nscenes, const BScene<T> *scenes, MgSettings ms,
                   size_t smem);
template <class T> cudaError_t b_tail_enable(size_t bytes);
// The coarse levels' descent (presmooth, sweeps, restrict per level) and
// ascent (post_black, sweeps, red sweep per level) as cooperative launches
// with grid barriers between passes; L.blocks must not exceed
// b_coarse_capacity (every block resident).
template <class T>
cudaError_t b_coarse_descend(const BLaunch &L, const BLevel<T> *levels, const CoarseLists &cl,
                             const BScene<T> *scenes, MgSettings ms);
template <class T>
cudaError_t b_coarse_ascend(const BLaunch &L, const BLevel<T> *levels, const CoarseLists &cl,
                            const BScene<T> *scenes, MgSettings ms, T alpha);
template <class T> int b_coarse_capacity(int sms);
template <class T>
cudaError_t b_direction(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                        const BScene<T> *scenes);
template <class T>
cudaError_t b_spmv(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n, const BScene<T> *scenes,
                   double *part);
template <class T>
cudaError_t b_update(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n, const BScene<T> *scenes,
                     double *part, int mode, BatchCounters *cnt);
template <class T>
cudaError_t b_refine_accumulate(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                                const BScene<T> *scenes);
template <class T>
cudaError_t b_refine_residual(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                              const BScene<T> *scenes, double *part, int initial, double residual, int max_iter,
                              double inner_rel, int inner_max, BatchCounters *cnt);

}  // namespace gbp
