// pn_batch.cpp -- batches of solvers advanced by shared launches.
//
// Members keep everything of their own (state, tables, sources, sensors,
// time, dt); a batch solve writes their argument blocks into one device array
// and launches, per step, one kernel per half step (table form) or one fused
// kernel (grid form) whose blocks walk the work tiles of all members.  The
// arithmetic of a member does not depend on the others, so a member's result
// is the same alone and in any batch.  pn_batch_solve returns when the steps
// are done (it waits for the GPU at the end of every signal-table chunk).
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>

#include "pn_noalloc.hpp"
#include "pn_solver.hpp"

// The launch sequence of one chunk, as far as a CUDA graph of it depends on it
// (kernel arguments are device pointers to the staged blocks plus the step).
struct ChunkSignature {
  int form, precision, n, shape, chunk, total0, total1, sym, tma;
  int rows;  // grid form: tile rows (also keeps the pointers 8-byte aligned with no padding bytes)
  const void *p[4];
  bool operator==(const ChunkSignature &o) const { return std::memcmp(this, &o, sizeof(*this)) == 0; }
};
static_assert(sizeof(ChunkSignature) == 10 * sizeof(int) + 4 * sizeof(void *), "no padding");

struct pn_batch {
  std::vector<pn_solver *> members;
  cudaStream_t stream = nullptr;
  // device staging of argument blocks and prefix tables
  void *d_args[2] = {nullptr, nullptr};  // table: vel / stress; grid: even / odd step parity
  int *d_start[2] = {nullptr, nullptr};
  size_t cap_args = 0, cap_start = 0;

  // autotuner: launch shape chosen per (form, precision, member-count and
  // work-size class), by timing the candidates on real steps
  std::map<std::tuple<int, int, int, int>, int> tuned;
  // launch shape of the last chunk (grid form: tile rows, z chunks per column
  // with 0 = the launcher's choice; table form: 0, resident blocks per SM)
  int last_rows = 0, last_shape = 0;
  // CUDA graph of the last chunk whose launch sequence repeated
  bool seen = false;
  ChunkSignature last{};
  cudaGraphExec_t exec = nullptr;
  ChunkSignature exec_sig{};
  int64_t graph_launches = 0, graph_captures = 0;
  // grid-form launch orders already built, by the members, their tile rows
  // and chunk lengths (built on the host: reused across calls; cleared when
  // members are added or removed)
  struct Order {
    std::vector<const void *> members;
    std::vector<int> kchunk;
    int rows = 0;
    std::vector<int> ids;
  };
  std::vector<Order> orders;

  ~pn_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    for (int k = 0; k < 2; k++) {
      if (d_args[k]) cudaFree(d_args[k]);
      if (d_start[k]) cudaFree(d_start[k]);
    }
  }
};

namespace {

int berr(int code, const std::string &m) { return pn::set_last_error(code, m); }

template <typename F>
int bguard(F &&f) {
  pn::set_last_error(PN_OK, "");
  try {
    return f();
  } catch (const pn::SetupError &e) {
    return berr(e.code, e.msg);
  } catch (const pn::CudaError &e) {
    (void)cudaGetLastError();
    return berr(PN_ERR_CUDA, std::string(e.what) + ": " + cudaGetErrorString(e.e));
  } catch (const std::exception &e) {
    return berr(PN_ERR_RUNTIME, e.what());
  }
}

void ensure_capacity(pn_batch *b, size_t args_bytes, size_t start_ints) {
  if (args_bytes > b->cap_args) {
    for (int k = 0; k < 2; k++) {
      if (b->d_args[k]) cudaFree(b->d_args[k]);
      b->d_args[k] = nullptr;
      pn::ck(cudaMalloc(&b->d_args[k], args_bytes), "batch args");
    }
    b->cap_args = args_bytes;
  }
  if (start_ints > b->cap_start) {
    for (int k = 0; k < 2; k++) {
      if (b->d_start[k]) cudaFree(b->d_start[k]);
      b->d_start[k] = nullptr;
      pn::ck(cudaMalloc(&b->d_start[k], start_ints * sizeof(int)), "batch tiles");
    }
    b->cap_start = start_ints;
  }
}

// where one batch call stages the argument blocks and tile prefixes its
// launches read: table form [0] velocity / [1] stress, grid form [0] even /
// [1] odd step parity
struct Staging {
  void *args[2];
  int *start[2];
};

// pn_batch_solve: the batch's own buffers, grown with cudaMalloc as needed
struct GrownStaging {
  pn_batch *b;
  Staging operator()(size_t args_bytes, size_t start_ints) const {
    ensure_capacity(b, args_bytes, start_ints);
    return Staging{{b->d_args[0], b->d_args[1]}, {b->d_start[0], b->d_start[1]}};
  }
};

// pn_batch_solve_noalloc: carved from the fixed device scratch (the caller
// has checked that the call fits)
struct ScratchStaging {
  unsigned char *base;
  static size_t round(size_t n) { return (n + 255) / 256 * 256; }
  static size_t bytes(size_t args_bytes, size_t start_ints) {
    return 2 * round(args_bytes) + 2 * round(start_ints * sizeof(int));
  }
  Staging operator()(size_t args_bytes, size_t start_ints) const {
    const size_t a = round(args_bytes), st = round(start_ints * sizeof(int));
    if (bytes(args_bytes, start_ints) > pn::kNoAllocScratchBytes)
      throw pn::SetupError{PN_ERR_INVALID, "batch staging exceeds the fixed scratch"};
    return Staging{{base, base + a}, {(int *)(base + 2 * a), (int *)(base + 2 * a + st)}};
  }
};

// steps all members can take with their current signal tables (may_alloc
// false: tables are refilled in place, never grown)
int32_t common_chunk(pn_batch *b, int32_t want, bool may_alloc = true) {
  int32_t chunk = want;
  for (pn_solver *s : b->members) {
    pn::ensure_signal_rows(s, chunk, may_alloc);
    if (!s->src.empty() && !s->sig_hold)
      chunk = (int32_t)std::min<int64_t>(chunk, s->sig_step0 + s->sig_rows - s->step);
  }
  return std::max<int32_t>(chunk, 1);
}

// ---- launch planning: autotuned shapes and graph replay -------------------
//
// A "shape" is how the work of one step is spread over the GPU; it never
// changes what a member computes (every node and cell is updated by one
// thread with the same arithmetic), only how fast:
//   table form  resident blocks per SM of the tile-walking kernels
//   grid form   tile rows (32 x 8 or, FP32 with the tensor-copy kernel, 32 x 16
//               block tiles: members are re-tiled to try them) x z chunks per
//               tile column (blocks = tiles x chunks)
// The first chunk of a new (form, precision, members, work) class long
// enough for it runs two steps with each candidate, twice in interleaved
// rounds, timed with CUDA events on the batch stream, and keeps the candidate
// with the fastest round for the rest of the chunk and for later chunks of the
// class (two rounds: one host-side hiccup does not decide the choice).  A chunk whose launch sequence equals the
// previous chunk's is captured as a CUDA graph and replayed from then on
// (work on a created stream only; the legacy default stream cannot be
// captured).  Neither runs in the allocation-free solve.
constexpr int kTableShapes[] = {8, 4, 16, 2};  // blocks per SM
constexpr int kGridChunkShapes[] = {0, 1, 2};  // 0: the launcher's choice; else chunks per column
constexpr int kGridRowShapes[] = {8, 16};       // tile rows, where the storage has them
constexpr int kTunePerShape = 2;               // timed steps per candidate and round
constexpr int kTuneRounds = 2;

int log2_class(int64_t v) { return v <= 1 ? 0 : (int)std::log2((double)v); }

template <typename Prepare, typename Launch>
void run_chunk(pn_batch *b, std::tuple<int, int, int, int> cls, int n_shapes, int32_t chunk, bool may_plan,
               ChunkSignature sig, int fallback, Prepare &&prepare, Launch &&launch) {
  int32_t k = 0;
  auto it = b->tuned.find(cls);
  int best = it == b->tuned.end() ? -1 : it->second;
  if (best < 0 && may_plan && n_shapes > 1 && chunk >= kTuneRounds * n_shapes * kTunePerShape + 1) {
    constexpr int kMaxShapes = 8;
    cudaEvent_t ev[kTuneRounds][2 * kMaxShapes];
    for (int r = 0; r < kTuneRounds; r++)
      for (int c = 0; c < 2 * n_shapes; c++) pn::ck(cudaEventCreate(&ev[r][c]), "tune event");
    for (int r = 0; r < kTuneRounds; r++)
      for (int c = 0; c < n_shapes; c++) {
        prepare(c);
        pn::ck(cudaEventRecord(ev[r][2 * c], b->stream), "tune event");
        for (int j = 0; j < kTunePerShape; j++) launch(c, k++);
        pn::ck(cudaEventRecord(ev[r][2 * c + 1], b->stream), "tune event");
      }
    pn::ck(cudaStreamSynchronize(b->stream), "tune sync");
    float best_ms = 0.f;
    for (int c = 0; c < n_shapes; c++) {
      float ms = 0.f;
      for (int r = 0; r < kTuneRounds; r++) {
        float m = 0.f;
        pn::ck(cudaEventElapsedTime(&m, ev[r][2 * c], ev[r][2 * c + 1]), "tune time");
        ms = r == 0 ? m : std::min(ms, m);
      }
      if (best < 0 || ms < best_ms) {
        best = c;
        best_ms = ms;
      }
    }
    for (int r = 0; r < kTuneRounds; r++)
      for (int c = 0; c < 2 * n_shapes; c++) cudaEventDestroy(ev[r][c]);
    b->tuned[cls] = best;
  }
  if (best < 0) best = fallback;
  const int units = prepare(best);  // work units of the shape (part of the launch sequence)
  if (k == 0 && may_plan && b->stream != nullptr) {
    sig.shape = best;
    sig.chunk = chunk;
    sig.total1 += units;
    if (b->exec && sig == b->exec_sig) {
      pn::ck(cudaGraphLaunch(b->exec, b->stream), "graph launch");
      b->graph_launches++;
      return;
    }
    if (b->seen && sig == b->last) {  // second time in a row: capture, then replay
      cudaGraph_t graph = nullptr;
      pn::ck(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "capture");
      try {
        for (; k < chunk; k++) launch(best, k);
      } catch (...) {
        cudaStreamEndCapture(b->stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
      }
      pn::ck(cudaStreamEndCapture(b->stream, &graph), "capture end");
      if (b->exec) cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
      const cudaError_t e = cudaGraphInstantiate(&b->exec, graph, 0);
      cudaGraphDestroy(graph);
      pn::ck(e, "graph instantiate");
      b->exec_sig = sig;
      b->graph_captures++;
      pn::ck(cudaGraphLaunch(b->exec, b->stream), "graph launch");
      b->graph_launches++;
      return;
    }
    b->seen = true;
    b->last = sig;
  }
  for (; k < chunk; k++) launch(best, k);
}

// per-member bookkeeping after `chunk` steps (time accumulated step by step,
// as solve() does)
void advance(pn_batch *b, int32_t chunk) {
  for (pn_solver *s : b->members) {
    for (int32_t k = 0; k < chunk; k++) s->time += s->dt;
    if (s->form == PN_FORM_GRID && (chunk & 1)) s->cur ^= 1;
    s->step += chunk;
    s->rec_count += chunk;
  }
}

template <typename T, typename Stage>
void solve_table(pn_batch *b, int32_t nsteps, int precision, const Stage &stage, bool may_alloc) {
  const int n = (int)b->members.size();
  std::vector<pn::VelArgs<T>> va(n);
  std::vector<pn::StressArgs<T>> sa(n);
  std::vector<int> vs(n + 1, 0), ss(n + 1, 0);
  int32_t done = 0;
  while (done < nsteps) {
    const int32_t chunk = common_chunk(b, nsteps - done, may_alloc);
    for (int m = 0; m < n; m++) {
      pn_solver *s = b->members[m];
      pn::table_args<T>(s, va[m], sa[m]);
      const int64_t nsig = (int64_t)s->src.size();
      if (nsig > 0) {
        const int64_t row0 = pn::sig_row(s, 0);
        va[m].sigval = (const T *)s->d_sig + row0 * nsig;
        va[m].sig_stride = (int32_t)nsig;
        va[m].sig_rows = (int32_t)(s->sig_rows - row0);
        sa[m].sigval = va[m].sigval;
        sa[m].sig_stride = va[m].sig_stride;
        sa[m].sig_rows = va[m].sig_rows;
      }
      va[m].rec_base = s->rec_count;
      vs[m + 1] = vs[m] + (s->mesh.n_nodes + pn::kTile - 1) / pn::kTile;
      ss[m + 1] = ss[m] + (s->mesh.n_cells + pn::kTile - 1) / pn::kTile;
    }
    const Staging g = stage(std::max(sizeof(pn::VelArgs<T>), sizeof(pn::StressArgs<T>)) * n, n + 1);
    pn::ck(cudaMemcpyAsync(g.args[0], va.data(), sizeof(pn::VelArgs<T>) * n, cudaMemcpyHostToDevice,
                           b->stream), "batch args");
    pn::ck(cudaMemcpyAsync(g.args[1], sa.data(), sizeof(pn::StressArgs<T>) * n, cudaMemcpyHostToDevice,
                           b->stream), "batch args");
    pn::ck(cudaMemcpyAsync(g.start[0], vs.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, b->stream),
           "batch tiles");
    pn::ck(cudaMemcpyAsync(g.start[1], ss.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, b->stream),
           "batch tiles");
    int dev = 0, sms = 1;
    pn::ck(cudaGetDevice(&dev), "device");
    pn::ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
    pn::BatchLaunch L;
    L.n_members = n;
    L.vel_args = g.args[0];
    L.str_args = g.args[1];
    L.vel_start = g.start[0];
    L.str_start = g.start[1];
    L.vel_tiles = vs[n];
    L.str_tiles = ss[n];
    // blocks walk the tiles: resident blocks per SM by the tuned shape, never more than tiles
    int staged = 0;
    auto shape = [&](int c) {
      staged = c;
      L.blocks_vel = std::min(vs[n], sms * kTableShapes[c]);
      L.blocks_str = std::min(ss[n], sms * kTableShapes[c]);
      return 0;
    };
    ChunkSignature sig{};
    sig.form = PN_FORM_TABLE;
    sig.precision = precision;
    sig.n = n;
    sig.total0 = vs[n];
    sig.total1 = ss[n];
    sig.p[0] = g.args[0];
    sig.p[1] = g.args[1];
    sig.p[2] = g.start[0];
    sig.p[3] = g.start[1];
    run_chunk(b, std::make_tuple((int)PN_FORM_TABLE, precision, log2_class(n), log2_class(vs[n] + ss[n])),
              (int)(sizeof(kTableShapes) / sizeof(int)), chunk, may_alloc, sig, 0, shape, [&](int c, int32_t k) {
                shape(c);
                pn::ck(pn::launch_table_batch(L, precision, k, b->stream), "batch step");
              });
    pn::ck(cudaStreamSynchronize(b->stream), "batch chunk");  // staging is reused next chunk
    b->last_rows = 0;
    b->last_shape = kTableShapes[staged];
    advance(b, chunk);
    done += chunk;
  }
}

template <typename T, typename Stage>
void solve_grid(pn_batch *b, int32_t nsteps, int precision, const Stage &stage, bool may_alloc) {
  const int n = (int)b->members.size();
  std::vector<pn::GridArgs<T>> ga[2] = {std::vector<pn::GridArgs<T>>(n), std::vector<pn::GridArgs<T>>(n)};
  std::vector<int> bs(n + 1, 0);
  std::vector<int> split(2 * (n + 1), 0);  // prefixes of the members' copies, then of their fix cells
  const int tx = pn::kGridTileX;
  int sym = 2;
  bool tma = true;  // the tensor-copy kernel when every member has its maps
  for (pn_solver *s : b->members) tma = tma && s->d_tmaps != nullptr;
  // launch shapes: (tile rows, z chunks per column) in a fixed order; the
  // untuned and the allocation-free calls keep the members' current tile rows
  bool same_rows = true;
  for (pn_solver *s : b->members) same_rows = same_rows && s->tile_rows == b->members.front()->tile_rows;
  if (!same_rows && !may_alloc)
    throw pn::SetupError{PN_ERR_INVALID, "batch members are tiled differently; one pn_batch_solve call re-tiles "
                                         "them"};
  const int rows0 = same_rows ? b->members.front()->tile_rows : pn::kGridTileRows;
  std::vector<std::pair<int, int>> shapes;
  int keep = 0;  // (rows0, the launcher's chunks)
  for (int rows : kGridRowShapes) {
    if (rows != pn::kGridTileRows && (!tma || !pn::grid_tma_rows_supported(precision, rows))) continue;
    for (int per : kGridChunkShapes) {
      if (rows == rows0 && per == 0) keep = (int)shapes.size();
      shapes.emplace_back(rows, per);
    }
  }
  // FP64 form: the per-block path choice when every member keeps its flags
  bool range_flags = tma && precision == PN_PREC_F64;
  for (pn_solver *s : b->members) range_flags = range_flags && s->d_rflags != nullptr;
  int32_t done = 0;
  while (done < nsteps) {
    const int32_t chunk = common_chunk(b, nsteps - done, may_alloc);
    // argument blocks of every member for shape c (tile rows; z chunks: 0 the
    // launcher's choice, else that many per column), both step parities,
    // staged; members are re-tiled first when the shape's rows differ
    Staging g{};
    int staged_shape = -1;
    // pn_batch_solve's launch order (the tensor-copy kernel): the blocks with
    // layers to march, longest first (stable: equal columns stay in member and
    // tile order, neighbours together); the staged prefix table holds it
    // after the members' block prefixes, sized for the shape with the most
    // blocks so that the staging is not reallocated between shapes.  The
    // allocation-free call keeps the plain numbering (no room in its scratch).
    const bool ordered = tma && may_alloc;
    std::vector<int> order;
    int listed = 0;  // blocks launched
    size_t start_ints = 2 * (n + 1);
    if (ordered) {
      size_t most = 0;
      for (auto &sh : shapes) {
        size_t blocks = 0;
        for (pn_solver *s : b->members) {
          const int kc = sh.second == 0 ? pn::grid_chunk_layers(precision, s->grid.nx, s->grid.ny, s->grid.nz, tma,
                                                                sh.first)
                                        : std::min(pn::kGridChunkMax, std::max(1, (s->grid.nz + sh.second - 1) /
                                                                                       sh.second));
          blocks += (size_t)(s->grid.nx / (tx - 1) + 1) * (s->grid.ny / (sh.first - 1) + 1) *
                    ((s->grid.nz + kc - 1) / kc);
        }
        most = std::max(most, blocks);
      }
      start_ints = std::max(start_ints, (size_t)(n + 1) + most);
    }
    auto prepare = [&](int c) {
      if (c == staged_shape) return listed;
      const int rows = shapes[c].first;
      bool retile = false;
      for (pn_solver *s : b->members) retile = retile || s->tile_rows != rows;
      if (retile) {
        if (!may_alloc) throw pn::SetupError{PN_ERR_INVALID, "re-tiling needs device allocation"};
        pn::ck(cudaStreamSynchronize(b->stream), "retile sync");  // queued steps read the old tables
        for (pn_solver *s : b->members)
          if (!pn::grid_set_tile_rows(s, rows))
            throw pn::SetupError{PN_ERR_INVALID, "member cannot take " + std::to_string(rows) + "-row tiles"};
      }
      for (int m = 0; m < n; m++) {
        pn_solver *s = b->members[m];
        pn::GridArgs<T> a;
        pn::grid_args<T>(s, a);
        const int64_t nsig = (int64_t)s->src.size();
        if (nsig > 0) {
          const int64_t row0 = pn::sig_row(s, 0);
          a.sigval = (const T *)s->d_sig + row0 * nsig;
          a.sig_stride = (int32_t)nsig;
          a.sig_rows = (int32_t)(s->sig_rows - row0);
        }
        a.rec = s->rec_count;
        const int per = shapes[c].second;
        a.kchunk = per == 0 ? pn::grid_chunk_layers(precision, a.nx, a.ny, a.nz, tma, rows)
                            : std::min(pn::kGridChunkMax, std::max(1, (a.nz + per - 1) / per));
        for (int p = 0; p < 2; p++) {  // step parity: buffers swap every step
          pn::GridArgs<T> q = a;
          const int in = s->cur ^ p, out = in ^ 1;
          q.tmaps = tma ? pn::grid_maps_for(s, in) : nullptr;
          for (int cc = 0; cc < 3; cc++) {
            q.V_in[cc] = (const T *)s->V[in][cc];
            q.V_out[cc] = (T *)s->V[out][cc];
          }
          for (int cc = 0; cc < 6; cc++) {
            q.S_in[cc] = (const T *)s->S[in][cc];
            q.S_out[cc] = (T *)s->S[out][cc];
          }
          ga[p][m] = q;
        }
        const int64_t blocks = (int64_t)(a.nx / (tx - 1) + 1) * (a.ny / (rows - 1) + 1) *
                               ((a.nz + a.kchunk - 1) / a.kchunk);
        bs[m + 1] = (int)(bs[m] + blocks);
        split[m + 1] = split[m] + a.n_copies;
        split[n + 1 + m + 1] = split[n + 1 + m] + a.n_fix;
      }
      listed = bs[n];
      const pn_batch::Order *cached = nullptr;
      if (ordered) {
        pn_batch::Order key;
        key.rows = rows;
        for (int m = 0; m < n; m++) {
          key.members.push_back(b->members[m]);
          key.kchunk.push_back(ga[0][m].kchunk);
        }
        for (const pn_batch::Order &o : b->orders)
          if (o.rows == key.rows && o.members == key.members && o.kchunk == key.kchunk) cached = &o;
        if (!cached) {
          if (b->orders.size() >= 8) b->orders.erase(b->orders.begin());
          b->orders.push_back(std::move(key));
        }
      }
      if (ordered && cached) {
        order = cached->ids;
        listed = (int)order.size();
      } else if (ordered) {
        // layers each block marches: its chunk of its tile column, up to the
        // column's top solid layer
        std::vector<std::pair<int, int>> work;  // (layers, block)
        work.reserve((size_t)bs[n]);
        for (int m = 0; m < n; m++) {
          pn_solver *s = b->members[m];
          const pn::GridArgs<T> &a = ga[0][m];
          const std::vector<int32_t> top = pn::grid_tile_tops(s->grid, rows);
          const int tiles = (int)top.size();
          for (int id = bs[m]; id < bs[m + 1]; id++) {
            const int local = id - bs[m], tile = local % tiles, k0 = local / tiles * a.kchunk;
            const int layers = std::min(std::min(top[(size_t)tile], a.nz), k0 + a.kchunk) - k0;
            // (a column's first chunk always runs: the FP64 form's blocks clear
            // their tile's flag word there)
            if (layers > 0 || k0 == 0) work.emplace_back(std::max(layers, 0), id);
          }
        }
        std::stable_sort(work.begin(), work.end(),
                         [](const std::pair<int, int> &x, const std::pair<int, int> &y) { return x.first > y.first; });
        order.resize(work.size());
        for (size_t q = 0; q < work.size(); q++) order[q] = work[q].second;
        listed = (int)order.size();
        b->orders.back().ids = order;
      }
      g = stage(sizeof(pn::GridArgs<T>) * n, start_ints);
      for (int p = 0; p < 2; p++)
        pn::ck(cudaMemcpyAsync(g.args[p], ga[p].data(), sizeof(pn::GridArgs<T>) * n, cudaMemcpyHostToDevice,
                               b->stream), "batch args");
      pn::ck(cudaMemcpyAsync(g.start[0], bs.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, b->stream),
             "batch blocks");
      if (ordered && listed > 0)
        pn::ck(cudaMemcpyAsync(g.start[0] + n + 1, order.data(), sizeof(int) * (size_t)listed,
                               cudaMemcpyHostToDevice, b->stream),
               "batch block order");
      pn::ck(cudaMemcpyAsync(g.start[1], split.data(), sizeof(int) * split.size(), cudaMemcpyHostToDevice,
                             b->stream), "batch split sites");
      staged_shape = c;
      return listed;
    };
    sym = 2;  // the most general symmetry class among the members
    for (pn_solver *s : b->members) sym = std::min(sym, s->sym);
    if (tma) {  // the cubic variant when every member has its 0.25/h folded in
      bool cubic = true;
      for (pn_solver *s : b->members) cubic = cubic && s->gfold != 1.0;
      if (cubic) sym |= 4;
    }
    int64_t work = 0;
    for (pn_solver *s : b->members) work += (int64_t)s->grid.nx * s->grid.ny * s->grid.nz / 1024;
    const auto key = std::make_tuple((int)PN_FORM_GRID, precision, log2_class(n), log2_class(work));
    // the allocation-free call keeps the tiling: a tuned shape only when its rows match
    int fallback = keep;
    if (!may_alloc) {
      auto it = b->tuned.find(key);
      if (it != b->tuned.end() && shapes[it->second].first == rows0) fallback = it->second;
    }
    prepare(fallback);
    ChunkSignature sig{};
    sig.form = PN_FORM_GRID;
    sig.precision = precision;
    sig.n = n;
    sig.sym = sym;
    sig.tma = tma ? 1 : 0;
    sig.p[0] = g.args[0];
    sig.p[1] = g.args[1];
    sig.p[2] = g.start[0];
    sig.p[3] = g.start[1];
    sig.rows = shapes[fallback].first;
    // (the allocation-free call looks up no tuned shape of its own: `fallback`)
    run_chunk(b, may_alloc ? key : std::make_tuple(-1, 0, 0, 0), (int)shapes.size(), chunk, may_alloc, sig,
              fallback, prepare,
              [&](int c, int32_t k) {
                prepare(c);
                pn::GridBatchLaunch L;
                L.n_members = n;
                L.args = g.args[k & 1];
                L.block_start = g.start[0];
                L.total_blocks = listed;
                L.order = ordered ? g.start[0] + n + 1 : nullptr;
                L.sym = sym;
                L.tile_rows = shapes[c].first;
                L.range_flags = range_flags ? 1 : 0;
                pn::ck(tma ? pn::launch_grid_tma_batch(L, precision, k, b->stream)
                           : pn::launch_grid_batch(L, precision, k, b->stream),
                       "batch step");
                if (split[n] > 0 || split[2 * n + 1] > 0) {
                  pn::GridSplitBatch F;
                  F.n_members = n;
                  F.args = g.args[k & 1];
                  F.copy_start = g.start[1];
                  F.fix_start = g.start[1] + n + 1;
                  F.total_copies = split[n];
                  F.total_fix = split[2 * n + 1];
                  pn::ck(pn::launch_grid_split_batch(F, precision, k, b->stream), "batch split sites");
                }
              });
    pn::ck(cudaStreamSynchronize(b->stream), "batch chunk");
    if (!range_flags)  // members stepped without their flags: FP64 path first when next alone
      for (pn_solver *s : b->members) pn::grid_reset_range_flags(s);
    b->last_rows = shapes[staged_shape].first;
    b->last_shape = shapes[staged_shape].second;
    advance(b, chunk);
    done += chunk;
  }
}

template <typename Stage>
void solve_members(pn_batch *b, int32_t nsteps, const Stage &stage, bool may_alloc) {
  const pn_solver *f = b->members.front();
  if (f->form == PN_FORM_GRID) {
    if (f->is_df64()) solve_grid<float2>(b, nsteps, f->precision, stage, may_alloc);
    else if (f->esz == 8) solve_grid<double>(b, nsteps, f->precision, stage, may_alloc);
    else solve_grid<float>(b, nsteps, f->precision, stage, may_alloc);
  } else {
    if (f->is_df64()) solve_table<float2>(b, nsteps, f->precision, stage, may_alloc);
    else if (f->esz == 8) solve_table<double>(b, nsteps, f->precision, stage, may_alloc);
    else solve_table<float>(b, nsteps, f->precision, stage, may_alloc);
  }
}

// device bytes one batch call stages (ScratchStaging layout)
size_t scratch_bytes(const pn_batch *b) {
  const size_t n = b->members.size();
  const pn_solver *f = b->members.front();
  size_t args = 0;
  const size_t starts = f->form == PN_FORM_GRID ? 2 * (n + 1) : n + 1;  // grid: block and split prefixes
  if (f->form == PN_FORM_GRID)
    args = f->is_df64() ? sizeof(pn::GridArgs<float2>) : f->esz == 8 ? sizeof(pn::GridArgs<double>)
                                                                       : sizeof(pn::GridArgs<float>);
  else
    args = f->is_df64() ? std::max(sizeof(pn::VelArgs<float2>), sizeof(pn::StressArgs<float2>))
         : f->esz == 8  ? std::max(sizeof(pn::VelArgs<double>), sizeof(pn::StressArgs<double>))
                        : std::max(sizeof(pn::VelArgs<float>), sizeof(pn::StressArgs<float>));
  return ScratchStaging::bytes(args * n, starts);
}

}  // namespace

extern "C" {

int pn_batch_create(pn_batch **out) {
  return bguard([&]() -> int {
    if (!out) return berr(PN_ERR_INVALID, "null output handle");
    *out = new pn_batch();
    return PN_OK;
  });
}

int pn_batch_add(pn_batch *b, pn_solver *m) {
  if (!b || !m) return berr(PN_ERR_INVALID, "null argument");
  for (pn_solver *x : b->members)
    if (x == m) return berr(PN_ERR_INVALID, "solver already in the batch");
  if (!b->members.empty()) {
    pn_solver *f = b->members.front();
    if (f->precision != m->precision || f->form != m->form)
      return berr(PN_ERR_INVALID, "batch members need one precision and one form");
  }
  if (m->precision == PN_PREC_F64_EXACT) return berr(PN_ERR_INVALID, "the exact FP64 form is not batched");
  if (m->has_mask_sources()) return berr(PN_ERR_INVALID, "window-mask sources need pn_solver_solve_signals");
  b->members.push_back(m);
  b->orders.clear();
  return PN_OK;
}

int pn_batch_remove(pn_batch *b, pn_solver *m) {
  if (!b || !m) return berr(PN_ERR_INVALID, "null argument");
  auto it = std::find(b->members.begin(), b->members.end(), m);
  if (it == b->members.end()) return berr(PN_ERR_INVALID, "solver not in the batch");
  b->members.erase(it);
  b->orders.clear();
  return PN_OK;
}

int pn_batch_size(pn_batch *b, int32_t *n) {
  if (!b || !n) return berr(PN_ERR_INVALID, "null argument");
  *n = (int32_t)b->members.size();
  return PN_OK;
}

int pn_batch_set_stream(pn_batch *b, void *stream) {
  return bguard([&]() -> int {
    if (!b) return berr(PN_ERR_INVALID, "null batch");
    pn::ck(cudaStreamSynchronize(b->stream), "stream switch");
    b->stream = (cudaStream_t)stream;
    return PN_OK;
  });
}

int pn_batch_solve(pn_batch *b, int32_t nsteps) {
  return bguard([&]() -> int {
    if (!b) return berr(PN_ERR_INVALID, "null batch");
    if (nsteps < 0) return berr(PN_ERR_INVALID, "negative step count");
    if (b->members.empty() || nsteps == 0) return PN_OK;
    for (pn_solver *s : b->members) {
      if (s->has_mask_sources()) return berr(PN_ERR_INVALID, "window-mask sources need pn_solver_solve_signals");
      pn::ck(cudaStreamSynchronize(s->stream), "member sync");  // members' own work first
      pn::refresh_sources(s);
    }
    solve_members(b, nsteps, GrownStaging{b}, true);
    return PN_OK;
  });
}

int pn_batch_solve_noalloc(pn_batch *b, int32_t nsteps) {
  return bguard([&]() -> int {
    if (!b) return berr(PN_ERR_INVALID, "null batch");
    if (nsteps < 0) return berr(PN_ERR_INVALID, "negative step count");
    if (b->members.empty() || nsteps == 0) return PN_OK;
    const size_t need = scratch_bytes(b);
    if (need > pn::kNoAllocScratchBytes)
      return berr(PN_ERR_INVALID, "pn_batch_solve_noalloc: " + std::to_string(b->members.size()) +
                                      " members need " + std::to_string(need) + " bytes of argument scratch, more "
                                      "than the fixed " + std::to_string(pn::kNoAllocScratchBytes) +
                                      " bytes; use pn_batch_solve or a smaller batch");
    for (size_t m = 0; m < b->members.size(); m++) {
      pn_solver *s = b->members[m];
      if (s->has_mask_sources()) return berr(PN_ERR_INVALID, "window-mask sources need pn_solver_solve_signals");
      if (s->src_dirty || (!s->src.empty() && s->sig_alloc_rows == 0))
        return berr(PN_ERR_INVALID, "pn_batch_solve_noalloc: member " + std::to_string(m) +
                                        " has sources whose device tables are not built yet; one pn_batch_solve "
                                        "or pn_solver_solve step builds them");
    }
    std::lock_guard<std::mutex> lock(pn::noalloc_call_lock());
    void *scratch = nullptr;
    pn::ck(pn::noalloc_scratch(&scratch), "scratch symbol address");
    for (pn_solver *s : b->members) pn::ck(cudaStreamSynchronize(s->stream), "member sync");
    try {
      solve_members(b, nsteps, ScratchStaging{(unsigned char *)scratch}, false);
    } catch (...) {
      // steps queued before the failure may still read the scratch: let them
      // finish before the lock lets another call restage it
      cudaStreamSynchronize(b->stream);
      throw;
    }
    return PN_OK;
  });
}

int pn_batch_plan_stats(pn_batch *b, int64_t *graph_launches, int64_t *graph_captures, int32_t *tuned_classes,
                        int32_t *tile_rows, int32_t *shape) {
  if (!b) return berr(PN_ERR_INVALID, "null batch");
  if (graph_launches) *graph_launches = b->graph_launches;
  if (graph_captures) *graph_captures = b->graph_captures;
  if (tuned_classes) *tuned_classes = (int32_t)b->tuned.size();
  if (tile_rows) *tile_rows = b->last_rows;
  if (shape) *shape = b->last_shape;
  return PN_OK;
}

int pn_batch_synchronize(pn_batch *b) {
  return bguard([&]() -> int {
    if (!b) return berr(PN_ERR_INVALID, "null batch");
    pn::ck(cudaStreamSynchronize(b->stream), "batch sync");
    pn::ck(cudaGetLastError(), "device error");
    for (pn_solver *m : b->members)
      if (const int rc = pn::device_check(m)) return rc;
    return PN_OK;
  });
}

int pn_batch_destroy(pn_batch *b) {
  if (!b) return PN_OK;
  cudaStreamSynchronize(b->stream);
  delete b;
  return PN_OK;
}

}  // extern "C"
