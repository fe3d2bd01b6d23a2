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

#include <cuda.h>
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
    // TMA descriptors of a staged fine level (STAGE_MAPS of them), or null
    const CUtensorMap *tmap;
    // tile classes (MgLevel::tcp, tcr), or null: every tile reads its arrays
    const T *tcp, *tcr;
};

// Staged fine-level kernels: a pair tile of 64 x 8 x 4 cells and the halo
// its stencil reads are copied into shared memory by TMA
// (cp.async.bulk.tensor) two tiles ahead of the compute. The boxes around a
// tile at (x0, y0, z0): HALO 72 x 10 x 6 from (x0-4, y0-1, z0-1) (x starts
// on a 16-byte boundary, hence 4 columns left), OWN 64 x 8 x 4 from the
// tile, CX 72 x 8 x 4 from (x0-4, y0, z0), CY 64 x 9 x 4 from (x0, y0-1, z0),
// CZ 64 x 8 x 5 from (x0, y0, z0-1), and XC 40 x 6 x 4 of the coarse grid
// from (x0/2-4, y0/2-1, z0/2-1) (the parents of the tile and its halo).
enum StageMap {
    SM_B_HALO, SM_INV_HALO, SM_X_HALO, SM_P_HALO, SM_CX, SM_CY, SM_CZ,
    SM_B_OWN, SM_INV_OWN, SM_DIAG_OWN, SM_XC, STAGE_MAPS
};
enum StageKind { STAGE_PRESMOOTH, STAGE_POST_BLACK, STAGE_RED_DOT, STAGE_SPMV, STAGE_KINDS };
constexpr int ST_TX = 64, ST_TY = 8, ST_TZ = 4;
// shared-memory bytes of one stage of each kind (two stages per block)
size_t stage_bytes(int kind);

// Per-scene state of the fine level.
template <class T> struct BScene {
    Grid g;
    T *x, *r, *z, *p, *q;  // PCG vectors (x: the correction in FP64 mode, d in mixed mode)
    // FP64 operator and refinement state
    Operator<double> A;
    // FP32 solver: the low floats of A against level 0's operator (A =
    // level 0 + lo within 2^-48), for the refinement's float-pair products;
    // null pointers otherwise
    Operator<float> lo;
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
    // the coarsest level in FP64 (x, b, inv, cx, cy, cz; MG_COARSEST_MAX
    // each), scratch of the batch runner
    double *c64;
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
    // test hook (gbp_debug_fail_wait), 0 in every ordinary solve: block
    // test_block of the kernels named by test_what (1: the cooperative
    // coarse kernels' grid barriers, 2: the TMA-staged fine kernels' tile
    // waits) leaves out its arrival / the copies of its first tile, and
    // every bounded wait polls at most test_polls times (0: the default)
    int test_what;
    int test_block;
    int test_polls;
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
    size_t tail_bytes = 0;
    // work lists as segments: pair[l] (pair tiles of level l), restrict[l]
    // (cell tiles of level l+1), fine (pair tiles of level 0), with their
    // item counts
    std::vector<std::vector<BSeg>> pair, restrict_;
    std::vector<BSeg> fine_pairs;
    std::vector<int> n_pair, n_restrict;
    int n_fine_pairs = 0;
    std::vector<int> fine_ref;           // level entry of each scene's fine level
};

// A launch of a batched kernel.
struct BLaunch {
    int blocks;
    cudaStream_t stream;
    int gate;
    const int *scene_of;  // scene of each level-table entry (reductions)
    BatchCounters *cnt;   // batch counters (idle and refinement checks)
    int occ;              // occupancy variant (4, 5 or 6 blocks per SM); 0: the precision's default
    int col;              // the list has 4-plane tiles: launch the gather-first column kernels
};

// Fine-level kernels whose occupancy variant the autotuner picks per batch.
enum BatchKernel { BK_PRESMOOTH, BK_RESTRICT, BK_POST_BLACK, BK_RED_DOT, BK_DIRECTION, BK_SPMV, BK_TUNED };

class BatchRunner {
public:
    BatchRunner() = default;
    ~BatchRunner() { release(); }
    BatchRunner(const BatchRunner &) = delete;
    BatchRunner &operator=(const BatchRunner &) = delete;

    // Uploads the plan (tables, lists) and sizes the partials. T = double
    // for the FP64 path, float for the inner solve of the mixed path.
    // staging (gbp_params.tma_staging): nonzero stages the FP32 fine levels
    // that qualify (the four stencil passes run TMA-staged there).
    template <class T> int build(const BatchPlan<T> &plan, int grid_blocks, int staging, cudaStream_t stream);
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
    // whether scene s's fine level runs TMA-staged kernels (any of the passes)
    bool scene_staged(int s) const {
        return stage_mask_ && s >= 0 && s < (int)staged_scene_.size() && staged_scene_[s];
    }
    int stage_mask() const { return stage_mask_; }
    // Test hook for the next solve only (see BatchCounters::test_what):
    // makes one block's bounded waits run out, polling at most `polls`.
    void set_wait_test(int what, int block, int polls) {
        test_what_ = what;
        test_block_ = block;
        test_polls_ = polls;
    }

private:
    int test_what_ = 0, test_block_ = 0, test_polls_ = 0;
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
    size_t tail_bytes_ = 0;
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
    int coarse_occ_ = 0;  // register variant of the cooperative kernels: 2 (bounds of 2 blocks per SM) or 0
    // fine levels split by staging: TMA-staged (FP32 levels that qualify) and
    // plain; each a segment list over pair tiles of level 0
    BSeg *d_fine_staged_ = nullptr, *d_fine_plain_ = nullptr;
    int n_fine_staged_ = 0, s_fine_staged_ = 0, n_fine_plain_ = 0, s_fine_plain_ = 0;
    CUtensorMap *d_tmaps_ = nullptr;
    std::vector<char> staged_scene_;
    int stage_mask_ = 0;  // bit k: pass k (StageKind) runs staged
    int occ_[BK_TUNED] = {};  // occupancy variant per tuned kernel (0: default)
    bool fine_col_ = false;    // some scene's fine level has 4-plane tiles of pairs (FP32)
    // a launch of tuned kernel bk (or -1: untuned) over `items` items
    template <class T> BLaunch launch_for(int bk, int items, cudaStream_t st, int gate) const;
    template <class T> int tune_occupancy(cudaStream_t st, const std::string &key);
public:
    // the chosen occupancy variant of tuned kernel bk (blocks of 256 threads per SM)
    template <class T> int occupancy(int bk) const { return occ_[bk] ? occ_[bk] : BatchOcc<T>::blocks; }
private:
    int sms_ = 0;
    template <class T> cudaError_t fine_pass(int kind, const gbp_params &p, cudaStream_t st, int gate);
    cudaGraphExec_t graph_ = nullptr;
    long long graph_key_ = -1;
    long long graph_nodes_ = 0;
    double inner_rel_ = 1e-3;
};



// Launch functions (batch_kernels.cu). `levels`, `scenes` and `segs` are
// device arrays.
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
cudaError_t b_tail(const BLaunch &L, const BTail<T> *tails, int nscenes, const BScene<T> *scenes, MgSettings ms);
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
// One staged fine-level pass (FP32) over the items of `segs`: presmooth,
// post_black (alpha), red_dot or spmv (partials in `part`). L.blocks <= SMs.
cudaError_t b_staged(int kind, const BLaunch &L, const BLevel<float> *levels, const BSeg *segs, int nseg, int n,
                     const BScene<float> *scenes, double *part, float alpha);
cudaError_t b_staged_enable();
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
cudaError_t b_refine_residual(const BLaunch &L, const BLevel<T> *levels, const BSeg *segs, int nseg, int n,
                              const BScene<T> *scenes, double *part, int initial, double residual, int max_iter,
                              double inner_rel, int inner_max, BatchCounters *cnt);

}  // namespace gbp
