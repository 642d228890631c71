// Application of multifrontal LU factors on the GPU, level by level or as a
// dataflow sweep (flow plans below).
//
// A FactorBank holds one or more factors (mf.hpp) concatenated node-wise.  Each
// factor is bound to a "RHS set": a list of right-hand sides that share the
// factor (e.g. electrons and holes of every instance when their mobilities
// are equal), so that every stored factor entry read from HBM is applied to
// all of them.  One kernel launch processes one tree level of every factor in
// the bank: wide nodes are split into row chunks handled by a CTA each
// (warp per row, coalesced row-major reads, warp-shuffle reduction); thin
// nodes (few columns) are stored column-major and applied thread-per-row,
// in warp-sized row chunks.  A bank built for many right-hand sides per set
// ("panel" banks) stores every block column-major and applies each node as a
// small dense GEMM: a CTA stages a chunk of columns of the right-hand sides
// (interleaved layout: a dof's values are contiguous) and of the block in
// shared memory, each warp accumulates a 4-row x (32 * RPL)-RHS register tile
// with lanes over right-hand sides, so every global access is coalesced.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "common.hpp"
#include "mf.hpp"

namespace pecs {

constexpr int kMaxSets = 4;
constexpr int kThinCols = 128;   // nodes with at most this many columns: thread per row
constexpr int kThinRows = 32;    // rows per warp item of a thin node (one per lane)
constexpr int kWideRows = 8;     // rows per CTA item of a wide node (one per warp)
constexpr int kTargetCtas = 152; // SMs of a GB300: levels with fewer wide items split rows
constexpr int kSolveThreads = 256;
constexpr size_t kSmemCap = 200 * 1024;  // dynamic shared memory budget per CTA
constexpr int kPanelMinRhs = 32;  // right-hand sides per set from which banks use the panel kernels

struct BankView {  // device pointers, passed by value to kernels
  const int* s;
  const int* m;
  const long long* goff;
  const long long* hoff;
  const int* own_off;
  const int* upd_off;
  const int* w_off;
  const int* cm_off;
  const int* own_idx;
  const int* upd_idx;
  const int* cmap_ptr;
  const int* cmap_idx;
  const int* node_set;
  const void* G;
  const void* H;
};

struct SetView {
  int nrhs;
  double* const* b;  // right-hand sides (read)
  double* const* y;  // forward result slots
  double* const* w;  // update-vector workspace (set_wtotal(set) doubles each)
  double* const* x;  // solutions (written)
};

struct SetsView {
  SetView set[kMaxSets];
};

// Interleaved layout: all right-hand sides of a set in one buffer, element
// (dof d, rhs r) at d * nrhs + r, so a dof's values are contiguous.
struct IlSetView {
  int nrhs;
  const double* b;
  double* y;
  double* w;  // update vectors, set_wtotal(set) x nrhs
  double* x;
};

struct IlSetsView {
  IlSetView set[kMaxSets];
};

// Interleaved layout with single-precision sweep vectors (FP32 factors on the
// panel path): b, y, update vectors and x are float -- they carry the FP32
// factors' results; refinement forms residuals in double-float and adds the
// correction to the solution outside the sweep.
struct IlSetViewF {
  int nrhs;
  const float* b;
  float* y;
  float* w;
  float* x;
};

struct IlSetsViewF {
  IlSetViewF set[kMaxSets];
};

// One level of the panel path: items (node, row0, row1, rows per tile), one
// CTA each; every item applies its rows of the node's block to a chunk of
// right-hand sides held in shared memory, lanes over right-hand sides.  Items
// are kept for row-tile caps 32, 16, 8 and 4; the launch picks one.
// One panel item: a row range of one node and everything about the node the
// kernel needs, so that a single round of loads starts it.
struct __align__(16) PanelItem {
  int4 a;  // node, row0, row1, rows per tile
  int4 b;  // s, m, RHS set, update-vector offset
  int4 c;  // block offset (low, high 32 bits), own-index offset, update-index offset
  int4 d;  // child-map pointer offset, first child-map entry, child-map entries, K part
  int4 e;  // split-K: first column, end column, tile (-1: no split), K parts of the tile
};

struct PanelTiles {
  int n_items = 0;
  int max_ri = 4;   // largest rows-per-tile of the items
  int min_ri = 32;  // smallest (< 32: column parts reduce in shared memory)
  int max_span = 0; // most columns one item covers (> the chunk width: double-buffered staging)
  DBuf<PanelItem> items;
};

// A tiling option of one panel level (see launch_panel_option).
struct PanelOption {
  int kind = -1;  // -1 untuned, 0 whole-row tiles, 1 split-K tiles, 2 leaf warps
  int cap_idx = 0;
  int rpl = 1;
};

struct PanelPlan {
  int max_k = 0;   // largest column count of the level's nodes
  int max_s = 1, max_f = 1;
  int cm_cap = 0;  // child-map entries staged per node (the level's largest, capped)
  int sc_rows[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // forward: child rows per chunk, per chunk size
  PanelTiles tiles[4];
  PanelTiles split;   // levels with long rows: 32-row tiles split along K (else empty)
  int split_tiles = 0;
  DBuf<int> counters;      // split-K: arrival counter per (tile, RHS chunk); reset by the last CTA
  DBuf<unsigned char> partials;  // split-K: [tile][part][32 rows][max RHS] partial products
  PanelTiles warp;    // leaf levels: one item per node, a warp each (else empty)
  int warp_rows = 0;  // leaf levels: most rows of a node
  PanelOption tuned;  // the autotuner's choice (kind -1: heuristic)
};

// A flow sweep of one direction (one persistent launch; solve.cu): work
// entries in topological order, the items they name, and per item the node
// counter it waits on (with its target) and the one it signals.
struct FlowPlan {
  int top = 0;       // tree levels it covers, from the root side (the rest: level launches)
  int rpl = 0;       // right-hand sides per lane (32 * rpl per chunk)
  int n_chunks = 0;  // right-hand-side chunks the entries cover
  int n_entries = 0;
  int kc_cap = 0, ds_rows = 0, ri_max = 0, sc_rows = 0, max_s = 1, max_f = 1, cm_cap = 0, nbuf = 1;
  int warp_max_k = 0, warp_rows_pad = 0;
  size_t smem = 0;
  int grid = 0;      // persistent CTAs (resident capacity, at most one per entry)
  DBuf<int4> entries, sync;
  DBuf<PanelItem> items;
};

// Host description of the factor tree a flow plan is built from (bank-wide
// node numbering; per node: sizes, RHS set, offsets, child-map pointer and
// parent, and the nodes of each height and depth).
struct FlowNodes {
  const std::vector<int>& s;
  const std::vector<int>& m;
  const std::vector<int>& node_set;
  const std::vector<int>& w_off;
  const std::vector<int>& own_off;
  const std::vector<int>& upd_off;
  const std::vector<int>& cm_off;
  const std::vector<int>& cmap_ptr;
  const std::vector<long long>& goff;
  const std::vector<long long>& hoff;
  const std::vector<int>& parent;
  std::vector<std::vector<int>> by_height, by_depth;
};

// A flow plan before upload: the launch shape, the items with their waits and
// signals ((wait counter or -1, target, signal counter or -1, 0)), and the
// entries in ticket order ((kind, first item, item count, RHS chunk)).
struct FlowPlanHost {
  bool ok = false;  // false: its staging does not fit in shared memory
  int n_chunks = 0;
  int kc_cap = 1, ds_rows = 1, ri_max = 4, sc_rows = 0, max_s = 1, max_f = 1, cm_cap = 0, nbuf = 1;
  int warp_max_k = 0, warp_rows_pad = 0;
  size_t smem = 0;
  std::vector<PanelItem> items;
  std::vector<int4> sync, entries;
};

// Builds one direction's flow plan over the `top` tree levels nearest the root
// (forward: the highest heights; backward: the smallest depths; top >= the
// level count: all of them) for rpl right-hand sides per lane and at most
// max_nrhs right-hand sides per set (host only; esz: bytes per value; kc_max:
// staged block columns per chunk; n_sm: multiprocessors to fill).
FlowPlanHost plan_flow(const FlowNodes& nd, bool forward, int top, int rpl, int max_nrhs, int kc_max, int esz,
                       int n_sm);

// The flow sweep of the few-right-hand-side path (one direction): the level
// plans' wide and thin items in topological order (solve.cu, k_rows_flow).
struct RowsFlowPlan {
  int n_entries = 0;
  DBuf<int4> entries, items, sync;
};

struct LevelPlan {
  int n_large = 0, n_thin = 0;
  DBuf<int4> items;   // wide nodes: (node, row0, row1, 0), one CTA each
  DBuf<int4> thin;    // thin nodes: (node, row0, row1, 0), one warp each
  int max_cols = 0;   // staged columns per large item
};

struct PanelTuning {
  int chunk = 0;     // staged block columns per chunk (0: 128 FP32, 64 FP64)
  int min_ctas = 0;  // CTAs a level must reach before shorter tiles are used (0: one per SM)
};

class FactorBank {
 public:
  // factors[i] is bound to RHS set i.  precision: PECS_PREC_FP64 or FP32_IR.
  // panel: store every block column-major and apply it with the panel
  // kernels (many right-hand sides per set, interleaved layout only).
  // max_nrhs: the most right-hand sides any set will carry (panel banks size
  // their split-K scratch with it)
  void build(const std::vector<const MfFactor*>& factors, int precision, bool panel = false,
             PanelTuning tuning = PanelTuning(), int max_nrhs = 0);
  // y = forward(b), x = backward(y); w is workspace.  All sets must be bound.
  void solve(const SetsView& sets, int max_nrhs, cudaStream_t st) const;
  void solve(const IlSetsView& sets, int max_nrhs, cudaStream_t st) const;
  void solve(const IlSetsViewF& sets, int max_nrhs, cudaStream_t st) const;
  int set_wtotal(int set) const { return set_wtotal_[set]; }
  int precision() const { return prec_; }
  long long entries() const { return entries_; }
  long long bytes() const { return bytes_; }
  int n_fwd_levels() const { return (int)fwd_.size(); }
  int n_bwd_levels() const { return (int)bwd_.size(); }
  int kernel_launches_per_solve() const;
  bool panel() const { return panel_; }
  // Panel banks: choose each level's tiling option by timing whole sweeps on
  // these right-hand sides (the sweep's outputs are garbage afterwards).
  // tuned_ms(): the tuned sweep's time.
  // flow_mode: 0 = the flow sweep when it times faster than the tuned levels,
  // 1 = the fastest flow sweep wherever one applies, -1 = levels only.
  void autotune(const IlSetsViewF& sets, int max_nrhs, cudaStream_t st, int reps = 3, int flow_mode = 0);
  void autotune(const IlSetsView& sets, int max_nrhs, cudaStream_t st, int reps = 3, int flow_mode = 0);
  // Few-right-hand-side banks: time the level sweep against the flow sweep on
  // these sets (a few sweeps each; outputs are garbage afterwards) and keep
  // the faster (flow_mode 0), the flow sweep (1) or the levels (-1).
  void tune_rows_flow(const IlSetsView& sets, int max_nrhs, cudaStream_t st, int flow_mode = 0, int reps = 3);
  bool rows_flow() const { return rows_flow_on_; }
  // Untuned banks: the flow sweep with the most right-hand sides per lane that
  // applies to these sets (the level sweep if none does).
  void force_flow(const IlSetsViewF& sets, int max_nrhs);
  void force_flow(const IlSetsView& sets, int max_nrhs);
  double tuned_ms() const { return tuned_ms_; }
  // Panel banks: right-hand sides per lane of the flow sweep in use (0: every
  // level its own launch), and the tree levels it covers from the root side.
  int flow_rpl() const { return flow_sel_ < 0 ? 0 : flow_cfg_[flow_sel_].rpl; }
  int flow_top() const {
    return rows_flow_on_ ? (int)fwd_.size() : (flow_sel_ < 0 ? 0 : flow_cfg_[flow_sel_].top);
  }
  // 1 if a flow sweep's wait ran out since the bank was built or the flag was
  // last cleared (that sweep's results were written as NaN); synchronises
  int flow_error(bool clear = false) const;
  // Diagnostic: the next forward flow sweep finds the first factor's root
  // counter far below its target, so that root's waits run out.
  void debug_arm_flow_stall() const;
  // Diagnostic: device time of each level launch of one sweep (forward levels,
  // then backward), CUDA events recorded between the launches, mean of reps
  // sweeps after one warm-up; the events keep consecutive levels from
  // overlapping, so the times are upper bounds of the in-sweep ones.
  std::vector<double> time_levels(const IlSetsViewF& sets, int max_nrhs, cudaStream_t st, int reps) const;
  int tune_launches() const { return tune_launches_; }

 private:
  int prec_ = PECS_PREC_FP64;
  int n_sets_ = 0;
  int set_wtotal_[kMaxSets] = {0, 0, 0, 0};
  long long entries_ = 0, bytes_ = 0;
  DBuf<int> s_, m_, own_off_, upd_off_, w_off_, cm_off_, own_idx_, upd_idx_, cmap_ptr_, cmap_idx_,
      node_set_;
  DBuf<long long> goff_, hoff_;
  DBuf<double> G64_, H64_;
  DBuf<float> G32_, H32_;
  std::vector<LevelPlan> fwd_, bwd_;
  std::vector<PanelPlan> pfwd_, pbwd_;
  bool panel_ = false;
  PanelTuning tune_;
  int parts_ld_ = 32;  // split-K scratch: right-hand sides per partial row
  int max_cols_ = 0, max_rb_ = 8;
  template <typename SVT>
  void solve_panel(const SVT& sets, int max_nrhs, cudaStream_t st) const;
  template <typename SVT>
  void autotune_panel(const SVT& sets, int max_nrhs, cudaStream_t st, int reps, int flow_mode);
  template <typename SVT>
  void force_flow_impl(const SVT& sets, int max_nrhs);
  template <typename SVT>
  int panel_rpl(const SVT& sets, int max_nrhs) const;
  double tuned_ms_ = 0.0;
  int tune_launches_ = 0;
  // flow sweeps built at creation: levels covered from the root side x staged
  // columns per chunk x right-hand sides per lane, both directions each
  struct FlowConfig {
    int top = 0, kc = 0, rpl = 0;
    FlowPlan plan[2];  // forward, backward
  };
  std::vector<FlowConfig> flow_cfg_;
  int flow_sel_ = -1;     // the configuration in use (-1: level launches only)
  DBuf<int> flow_state_;  // [2][nodes] counters, 2 tickets, error flag
  int n_nodes_ = 0;
  int stall_node_ = -1;  // the first factor's root (debug_arm_flow_stall)
  RowsFlowPlan rows_flow_plan_[2];
  bool rows_flow_on_ = false;
  int solve_rb(int max_nrhs) const;
  template <typename SV>
  void solve_rows_flow(const SV& sets, int max_nrhs, cudaStream_t st) const;
  void release_unused_flow();
  template <typename SVT>
  bool flow_ok(const SVT& sets, int max_nrhs, int cfg) const;
  template <typename SVT>
  void solve_flow(const SVT& sets, int max_nrhs, int cfg, cudaStream_t st) const;
  BankView view() const;
  template <typename SV>
  void solve_impl(const SV& sets, int max_nrhs, cudaStream_t st) const;
};

}  // namespace pecs
