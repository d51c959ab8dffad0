// Host runtime of the GB300 pressure-projection step: the C ABI of
// include/vfs_gpu.h, grid and multigrid-hierarchy setup, the V-cycle, the
// FP64 flexible GMRES driver and the whole projection step.
//
// The reference runs the same sequence on the CPU through PETSc and HYPRE
// (solvers.c:871-931, poisson_hypre.c:580-771, mhv_poisson.c:2121-2359).
// Here every array lives in HBM, every loop is a kernel, and the Krylov
// scalars stay on the device: the host only enqueues launches and reads one
// status word per iteration, one iteration behind, so the GPU never waits for
// the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "mg_group.h"
#include "mg_tiles.cuh"
#include "mg_stage.h"
#include "vfs_common.cuh"
#include "vfs_gpu.h"
#include "vfs_kernels.h"
#include "vfs_proj.h"

using namespace vfs;

std::atomic<unsigned long long> vfs::g_launches{0};

namespace {

// CUDA-event probe around every launch of one kernel of the finest level, or
// (VFS_PROBE_ALL) around every instrumented launch of a step, timed on the
// stream the kernel runs on, with its algorithmic bytes: the compulsory HBM
// reads and writes of the launch (operands once, results once).
struct ProbeRec {
  const char* name;
  int level;
  int ev;  // index of the start event
  double bytes;
  double ms = 0.;  // filled by vfs_probe_end
};
struct Probe {
  int kind = 0;  // VFS_PROBE_*
  std::vector<cudaEvent_t> ev;
  int used = 0;
  double bytes = 0.;
  unsigned long long launches = 0;
  std::vector<ProbeRec> recs;
  // a probe kind k is open; launches issued into a capturing stream (a batch
  // graph) are not probed: their events would become graph nodes
  bool wants(int k, cudaStream_t s) const {
    if (kind == 0 || (kind != k && kind != VFS_PROBE_ALL)) return false;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone;
  }
  bool begin(cudaStream_t s) {
    if (used + 2 > (int)ev.size()) return false;
    cudaEventRecord(ev[used], s);
    return true;
  }
  void end(cudaStream_t s, double b, const char* name = "", int level = -1, int count = 1) {
    cudaEventRecord(ev[used + 1], s);
    recs.push_back({name, level, used, b});
    used += 2;
    bytes += b;
    launches += count;
  }
};
Probe g_probe;

// Probe scope of one launcher call (kind k, or any under VFS_PROBE_ALL).
struct Probed {
  bool on;
  cudaStream_t s;
  const char* name;
  int level;
  double bytes;
  Probed(int k, cudaStream_t s_, const char* n, int l, double b) : s(s_), name(n), level(l), bytes(b) {
    on = g_probe.wants(k, s) && g_probe.begin(s);
  }
  ~Probed() {
    if (on) g_probe.end(s, bytes, name, level);
  }
};

// VFS_DEBUG_SYNC=1: synchronise after every launch stage of the solve and
// report the first stage that leaves a CUDA error (a self-check for faults).
const bool g_debug = [] {
  const char* e = getenv("VFS_DEBUG_SYNC");
  return e && e[0] == '1';
}();
int g_debug_err = 0;
void dbg(const char* stage, int level, int rc, cudaStream_t s) {
  if (!g_debug || g_debug_err) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) return;
  cudaError_t e = rc ? (cudaError_t)rc : cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_debug_err = (int)e;
    fprintf(stderr, "VFS_DEBUG_SYNC: %s (level %d) -> %s\n", stage, level, cudaGetErrorString(e));
  }
}

constexpr int MAXLEV = 12;
constexpr int MAXRESTART = 64;
constexpr int DENSE_MAX = 8192;  // largest coarsest level solved by a dense inverse

struct Level {
  Dims d{};
  size_t N = 0;
  double* coor = nullptr;
  double* nvert = nullptr;
  double* M = nullptr;
  double* coef = nullptr;
  double* mcoef = nullptr;
  float* mcoef32 = nullptr;
  float* lf32 = nullptr;   // y-line Thomas pivots 1/m
  float* rw32 = nullptr;   // restriction weights max(0, 1 - nvert)
  double* rw64 = nullptr;
  double* lf64 = nullptr;
  unsigned mask = 0;
  uint8_t* pcode = nullptr;
  float* x32[2] = {nullptr, nullptr};
  float* b32 = nullptr;
  double* x64[2] = {nullptr, nullptr};
  double* b64 = nullptr;
  double* Binv = nullptr;
  float* Binv32 = nullptr;
  int nco = 0;
  // FP16 diagonal-normalised operator of the FP32 multigrid (mg_half)
  __half* hcoef = nullptr;  // [19][hslot] (hidx layout)
  float* lfh = nullptr;     // its y-line pivots (0 on non-fluid rows)
  float* rwh = nullptr;     // its restriction weights (levels >= 1)
  float* dinvh = nullptr;   // finest level: 1 / D (input scaling)
  float* dvalh = nullptr;   // coarsest level: D (dense-solve scaling)
  // face form of the FP32 multigrid operator (mg_half = 0): +i / +k faces
  // (normal, cross weight), +j face, aj, cross-term code bits; on levels
  // with i-j or j-k cross terms also their weights (ffc)
  float2* ffi = nullptr;
  float2* ffk = nullptr;
  float* ffj = nullptr;
  float* faj = nullptr;
  float4* ffc = nullptr;
};

struct Grid {
  Dims d{};
  int L = 1, si = 0, sj = 0, sk = 0, immersed = 0;
  Level lev[MAXLEV];
  double* pd = nullptr;
  double* pw = nullptr;     // projection face weights (9, see launch_proj_weights)
  uint16_t* pc = nullptr;   // projection cross-term codes
  double* minv = nullptr;   // per-cell inverse metric / 2 (9, row-major), Contra2Cart
  uint8_t* nb8 = nullptr;   // nvert as bytes when all are integers in [0, 127], else null
  uint8_t* nb8_buf = nullptr;  // storage behind nb8
  double* mtmp = nullptr;   // metric formation scratch (9 N)
  double* u = nullptr;      // SoA Ucont: x | y | z
  double* ustar = nullptr;  // SoA resident U*
  double* p = nullptr;
  double* phi = nullptr;
  double* b = nullptr;
  double* bs = nullptr;     // aj-scaled right-hand side of the outer solve
  double dt = 0.04, st_ = 1.0, coeff = 1.0;  // of the last right-hand side
  double* ucat = nullptr;   // AoS
  double* aos = nullptr;    // AoS staging
  int m = 0;
  double* V = nullptr;
  double* w = nullptr;
  float* Z32 = nullptr;
  double* Z64 = nullptr;
  KrylovState* st = nullptr;
  double* starr = nullptr;
  double* parts = nullptr;
  double* scal = nullptr;   // small device scalars (sums, divmax)
  int* hstat = nullptr;     // pinned: done, epoch of the last status copy
  KrylovState* hk = nullptr;  // pinned copy of the Krylov state (convergence check)
  double* hv = nullptr;     // pinned: ||r||, max |r|, max |div u|
  int epoch = 0;            // solve rounds started on this grid
  cudaEvent_t ev_chk = nullptr, ev_done = nullptr, ev_pend = nullptr;
  cudaStream_t cs = nullptr;  // copy stream: host transfers that overlap the step
  cudaEvent_t ev_pin = nullptr, ev_p = nullptr, ev_u = nullptr, ev_cs = nullptr, ev_uin = nullptr;
  long long busy = 0;       // ticket of the request in flight on this grid (serving)
  cudaStream_t s = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  bool lhs = false;
  bool solo = false;  // the grid's solve runs alone (set by the driver before it issues work)
  bool half_ok = true;  // the FP16 operator represents every level (else mg_half runs the FP32 one)
  int ncomp = 1;         // connected fluid regions of the finest level
  int ncomp_c = 1;       // of the coarsest level
  int* comp = nullptr;   // finest-level region labels (device), when ncomp > 1
  cudaGraphExec_t ig_exec = nullptr;  // captured Arnoldi iteration
  int ig_prec = -1, ig_nu1 = -1, ig_nu2 = -1, ig_orth = -1, ig_cols = -1, ig_nu1c = -2, ig_nu2c = -2, ig_half = -1, ig_solo = -1;
  int ig_smoother = -1, ig_stage = -1;
  double ig_cheb_hi = 0., ig_cheb_ratio = 0.;
  unsigned long long ig_kernels = 0;  // kernels per replay
  double ig_omega = 0.;
  double nfluid = 0.;  // fluid interior cells of the finest level
  size_t bytes = 0;
  std::vector<void*> allocs;
  Ucont U() const { size_t N = ncell(d); return Ucont{u, u + N, u + 2 * N}; }
};

}  // namespace

struct vfs_job_box;  // a serving request (defined with the solve jobs)

struct vfs_ctx {
  int device = 0;
  cudaStream_t s0 = nullptr;  // batch stream (ticks of the batch graph)
  int max_inflight = 16;      // serving slots
  long long next_ticket = 1;
  std::map<long long, std::unique_ptr<vfs_job_box>> inflight;  // serving requests by ticket
  std::vector<cudaEvent_t> marks;  // vfs_mark slots
  size_t budget = 0, used = 0;
  std::map<int, Grid*> grids;
  int next_id = 1;
  std::string err;
};

namespace {

int fail(vfs_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}
int cuda_fail(vfs_ctx* c, cudaError_t e, const char* where) {
  return fail(c, VFS_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define CK(expr)                                             \
  do {                                                       \
    cudaError_t _e = (cudaError_t)(expr);                    \
    if (_e != cudaSuccess) return cuda_fail(ctx, _e, #expr); \
  } while (0)

// Connected regions of the fluid cells through shared faces, periodic wrap
// included: labels 0..K-1 in the order of each region's first cell (cell
// index order), -1 on other cells; returns K.  A grid that bodies cut
// apart has one constant null vector per region; the reference finds the
// two-region case of a k-blocked grid with FullyBlocked (poisson.c:1918-1998)
// and splits its null space at the first blocked k of each column
// (poisson.c:819-873).
int fluid_regions(const Dims& d, const std::vector<char>& fluid, std::vector<int>& label) {
  const size_t N = ncell(d);
  std::vector<int> parent(N, -1);
  auto find = [&](int a) {
    while (parent[a] != a) {
      parent[a] = parent[parent[a]];
      a = parent[a];
    }
    return a;
  };
  auto unite = [&](int a, int b) {
    a = find(a);
    b = find(b);
    if (a != b) parent[std::max(a, b)] = std::min(a, b);
  };
  for (size_t c = 0; c < N; c++)
    if (fluid[c]) parent[c] = (int)c;
  for (int k = 1; k < d.mz - 1; k++)
    for (int j = 1; j < d.my - 1; j++)
      for (int i = 1; i < d.mx - 1; i++) {
        const size_t c = cidx(d, i, j, k);
        if (!fluid[c]) continue;
        const int in = (i == d.mx - 2) ? (d.ip ? 1 : -1) : i + 1;
        const int jn = (j == d.my - 2) ? (d.jp ? 1 : -1) : j + 1;
        const int kn = (k == d.mz - 2) ? (d.kp ? 1 : -1) : k + 1;
        if (in > 0 && fluid[cidx(d, in, j, k)]) unite((int)c, (int)cidx(d, in, j, k));
        if (jn > 0 && fluid[cidx(d, i, jn, k)]) unite((int)c, (int)cidx(d, i, jn, k));
        if (kn > 0 && fluid[cidx(d, i, j, kn)]) unite((int)c, (int)cidx(d, i, j, kn));
      }
  label.assign(N, -1);
  std::vector<int> id(N, -1);
  int K = 0;
  for (size_t c = 0; c < N; c++) {
    if (parent[c] < 0) continue;
    const int r = find((int)c);
    if (id[r] < 0) id[r] = K++;
    label[c] = id[r];
  }
  return K;
}

template <typename T>
int galloc(vfs_ctx* ctx, Grid& g, T** out, size_t count) {
  const size_t bytes = count * sizeof(T);
  if (ctx->budget && ctx->used + bytes > ctx->budget)
    return fail(ctx, VFS_ERR_NOMEM, "HBM budget exceeded (" + std::to_string(ctx->used + bytes) + " > " +
                                        std::to_string(ctx->budget) + " bytes)");
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, VFS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  // Zero on the grid's own stream: a plain cudaMemset runs on the legacy
  // default stream, which does not order against the grid's non-blocking
  // stream, and could land after later writes (e.g. the Krylov state copy).
  e = cudaMemsetAsync(p, 0, bytes ? bytes : 16, g.s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync");
  g.allocs.push_back(p);
  g.bytes += bytes;
  ctx->used += bytes;
  *out = (T*)p;
  return VFS_OK;
}
#define GA(ptr, count)                                  \
  do {                                                  \
    int _r = galloc(ctx, g, &(ptr), (size_t)(count));   \
    if (_r) return _r;                                  \
  } while (0)

void grid_free(vfs_ctx* ctx, Grid* g) {
  if (g->s) cudaStreamSynchronize(g->s);
  for (void* p : g->allocs) cudaFree(p);
  if (ctx) ctx->used -= std::min(ctx->used, g->bytes);
  if (g->ig_exec) cudaGraphExecDestroy(g->ig_exec);
  if (g->hstat) cudaFreeHost(g->hstat);
  if (g->hk) cudaFreeHost(g->hk);
  if (g->hv) cudaFreeHost(g->hv);
  for (cudaEvent_t e : {g->ev_chk, g->ev_done, g->ev_pend, g->ev_pin, g->ev_p, g->ev_u, g->ev_cs, g->ev_uin})
    if (e) cudaEventDestroy(e);
  if (g->cs) {
    cudaStreamSynchronize(g->cs);
    cudaStreamDestroy(g->cs);
  }
  for (auto& e : g->ev) if (e) cudaEventDestroy(e);
  if (g->t0) cudaEventDestroy(g->t0);
  if (g->t1) cudaEventDestroy(g->t1);
  if (g->s) cudaStreamDestroy(g->s);
  delete g;
}

Grid* get_grid(vfs_ctx* ctx, int id) {
  auto it = ctx->grids.find(id);
  return it == ctx->grids.end() ? nullptr : it->second;
}

// Entry points that read or write a grid's device state refuse while a
// submitted request is in flight on it (its job owns the grid's buffers and
// stream until vfs_poll returns it).
int check_idle(vfs_ctx* ctx, const Grid* g) {
  return g->busy ? fail(ctx, VFS_ERR_BUSY, "the grid has a request in flight (vfs_poll it first)") : VFS_OK;
}

int coarse_n(int n) { return n / 2; }

template <typename T> T* mcoef_of(Level& L);
template <> float* mcoef_of<float>(Level& L) { return L.mcoef32; }
template <> double* mcoef_of<double>(Level& L) { return L.mcoef; }
template <typename T> T** xbuf(Level& L);
template <> float** xbuf<float>(Level& L) { return L.x32; }
template <> double** xbuf<double>(Level& L) { return L.x64; }
template <typename T> T*& bbuf(Level& L);
template <> float*& bbuf<float>(Level& L) { return L.b32; }
template <> double*& bbuf<double>(Level& L) { return L.b64; }
template <typename T> T* binv(Level& L);
template <> float* binv<float>(Level& L) { return L.Binv32; }
template <> double* binv<double>(Level& L) { return L.Binv; }

template <typename T>
OpView<T> mgview(Level& L, const int* skip) {
  return OpView<T>{L.d, mcoef_of<T>(L), L.mask, skip};
}

// The multigrid level data in use: the FP16 normalised operator's pivots,
// weights and scales when half is set (FP32 multigrid only), else the
// level's own.
template <typename T> T* lf_sel(Level& L, bool half);
template <> float* lf_sel<float>(Level& L, bool half) { return half ? L.lfh : L.lf32; }
template <> double* lf_sel<double>(Level& L, bool) { return L.lf64; }
template <typename T> T* rw_sel(Level& L, bool half);
template <> float* rw_sel<float>(Level& L, bool half) { return half ? L.rwh : L.rw32; }
template <> double* rw_sel<double>(Level& L, bool) { return L.rw64; }
template <typename T> T* dsc_sel(Level& L, bool half);
template <> float* dsc_sel<float>(Level& L, bool half) { return half ? L.dvalh : nullptr; }
template <> double* dsc_sel<double>(Level&, bool) { return nullptr; }
template <typename T> const float* dinv_sel(Level& L, bool half);
template <> const float* dinv_sel<float>(Level& L, bool half) { return half ? L.dinvh : nullptr; }
template <> const float* dinv_sel<double>(Level&, bool) { return nullptr; }
template <typename T>
OpView<T> mgview(Level& L, const int* skip, bool half, bool face = false) {
  OpView<T> A = mgview<T>(L, skip);
  if (sizeof(T) == 4 && half) A.hcoef = L.hcoef;
  if (sizeof(T) == 4 && !half && face) {
    A.ffi = L.ffi;
    A.ffk = L.ffk;
    A.ffj = L.ffj;
    A.faj = L.faj;
    if ((L.mask & ~0x7807Fu) != 0u) A.ffc = L.ffc;  // i-j or j-k cross terms: the general face form
  }
  return A;
}
// The face form of a level fits the 11-slot set (no i-j or j-k cross terms).
bool face_level(const Level& L) { return (L.mask & ~0x7807Fu) == 0u; }
// Operator bytes a face-form cell streams in a sweep (x != 0, or from a zero
// guess): the 11-slot form's 5 face weights and aj (24), plus on the general
// form the 4 cross weights (16); from a zero guess the j faces and aj (8),
// or aj and the assembled SP and NP (12).
template <typename T>
double face_sweep_bytes(const OpView<T>& A, bool x_nonzero) {
  if (A.ffc) return x_nonzero ? 40.0 : 12.0;
  return x_nonzero ? 24.0 : 8.0;
}

template <typename T>
int ensure_mg(vfs_ctx* ctx, Grid& g) {
  for (int l = 0; l < g.L; l++) {
    Level& L = g.lev[l];
    T** x = xbuf<T>(L);
    if (!x[0]) {
      GA(x[0], L.N);
      GA(x[1], L.N);
      GA(bbuf<T>(L), L.N);
    }
  }
  return VFS_OK;
}

int ensure_krylov(vfs_ctx* ctx, Grid& g, int m, int prec) {
  const size_t N = ncell(g.d);
  if (g.m < m) {
    if (g.m) return fail(ctx, VFS_ERR_ARG, "restart length cannot grow after the first solve of a grid");
    GA(g.V, (size_t)(m + 1) * N);
    GA(g.w, N);
    g.m = m;
    GA(g.starr, (size_t)(m + 1) * m + 7 * (m + 2));
  }
  if (prec == VFS_MIXED && !g.Z32) GA(g.Z32, (size_t)g.m * N);
  if (prec == VFS_FP64 && !g.Z64) GA(g.Z64, (size_t)g.m * N);
  return VFS_OK;
}

// ---------------------------------------------------------------------------
// V-cycle from a zero initial guess on level l: approximately solves
// A_l x = b; xa / xb are the level's ping-pong buffers; returns the buffer
// that holds the result.
// ---------------------------------------------------------------------------
constexpr int MAXSWEEP = 64;  // smoothing sweeps per level and side

struct MGCfg {
  int nu1, nu2, ncoarse;
  double omega, omega_c;
  double wf[2][MAXSWEEP];  // damping of the finest level's sweeps: [0] pre, [1] post
  double wc[2][MAXSWEEP];  // of the coarser levels' sweeps
  double w(int l, int post, int q) const { return (l == top ? wf : wc)[post][q]; }
  int cols;        // smoother columns per block (0 = automatic)
  int nu1c, nu2c;  // sweeps on the levels below the finest
  int top;         // index of the finest level
  bool half;       // FP16 normalised operator (FP32 multigrid only)
  bool face;       // FP32 face form on 11-slot levels (FP32 multigrid only)
  bool solo;       // the grid's solve runs alone
  int stage;       // how the finest face-form sweeps stage their operands (SweepStage)
  int pre(int l) const { return l == top ? nu1 : nu1c; }
  int post(int l) const { return l == top ? nu2 : nu2c; }
};

int popcount(unsigned m) {
  int c = 0;
  for (; m; m &= m - 1) c++;
  return c;
}
size_t n_interior(const Dims& d) { return (size_t)(d.mx - 2) * (d.my - 2) * (d.mz - 2); }

// A full smoothing sweep (x != 0) streams the active coefficient slots, x,
// b, the line pivots 1/m and writes x: (slots + 4) words per interior cell.
template <typename T>
void smooth_probed(int l, const OpView<T>& A, const T* lf, const T* xi, const T* b, T* xo, T omega, int cols, bool solo,
                   cudaStream_t s, int stage = STAGE_REGS) {
  // x != 0: the coefficient slots (FP16 or T), x, b and 1/m read, x written;
  // from a zero guess: the centre (not with the FP16 operator), SP and NP
  // slots, b and 1/m read, x written
  // face form: the 5 face weights and aj with the code bits (24 bytes) instead
  // of the slots; from a zero guess the j faces and aj (8 bytes)
  const double slot_bytes = A.hcoef ? 2.0 : (double)sizeof(T);
  const double op_bytes = A.ffi ? face_sweep_bytes(A, xi != nullptr)
                                 : (xi ? slot_bytes * popcount(A.mask) : slot_bytes * (A.hcoef ? 2 : 3));
  const double bytes = (double)n_interior(A.d) * (op_bytes + (xi ? 4.0 : 3.0) * sizeof(T));
  int rc;
  {
    Probed pr(VFS_PROBE_ALL, s, xi ? "k_smooth" : "k_smooth (zero guess)", l, bytes);
    rc = launch_smooth<T>(A, lf, xi, b, xo, omega, s, cols, solo, stage);
  }
  dbg("smooth", l, rc, s);
}

// VFS_PROBE_SMOOTH: one event pair around each run of consecutive full
// sweeps (x != 0) of the finest level, so that the event overhead is shared
// by the run's launches; bytes and launches counted per sweep.
struct SweepRun {
  bool on = false;
  cudaStream_t s = nullptr;
  int n = 0;
  double bytes = 0.;
  void add(bool probe, cudaStream_t s_, double b) {
    if (!probe) return;
    if (!on) {
      s = s_;
      on = g_probe.wants(VFS_PROBE_SMOOTH, s) && g_probe.begin(s);
    }
    if (on) {
      n++;
      bytes += b;
    }
  }
  void close() {
    if (on && n) g_probe.end(s, bytes, "k_smooth (run)", -1, n);
    on = false;
    n = 0;
    bytes = 0.;
  }
};

// Number of buffer writes of a level's schedule (smoothing sweeps, plus the
// prolongation when no pre-sweep wrote first): the result lands in
// bufs[(writes - 1) & 1], so the caller's first buffer is swapped in when
// needed to make the V-cycle's result always land in xa.
int level_writes(const Grid& g, int l, const MGCfg& c) {
  if (l == 0) return g.lev[0].Binv ? 1 : c.ncoarse;
  return c.pre(l) + (c.pre(l) == 0 ? 1 : 0) + c.post(l);
}

template <typename T>
T* vcycle(Grid& g, int l, T* b, T* xa, T* xb, const MGCfg& c, const int* skip, cudaStream_t s) {
  Level& L = g.lev[l];
  const bool half = sizeof(T) == 4 && c.half;
  const bool face = sizeof(T) == 4 && !half && c.face;
  OpView<T> A = mgview<T>(L, skip, half, face);
  T* lf = lf_sel<T>(L, half);
  const int W = level_writes(g, l, c);
  T* bufs[2] = {xa, xb};
  if (((W - 1) & 1) == 1) std::swap(bufs[0], bufs[1]);
  if (l == 0) {
    if (binv<T>(L)) {
      Probed pr(VFS_PROBE_ALL, s, "k_coarse_gemv", l, ((double)L.nco * L.nco + 2.0 * L.nco) * sizeof(T));
      dbg("coarse_gemv", l, launch_coarse_gemv<T>(L.d, binv<T>(L), L.nco, b, bufs[0], dsc_sel<T>(L, half), skip, s),
          s);
      return bufs[0];
    }
    T* cur = nullptr;
    for (int q = 0; q < c.ncoarse; q++) {
      T* o = bufs[q & 1];
      smooth_probed<T>(l, A, lf, cur, b, o, (T)c.omega_c, c.cols, c.solo, s);
      cur = o;
    }
    return cur;
  }
  int q = 0;
  T* cur = nullptr;
  const bool run_probe = g_probe.kind == VFS_PROBE_SMOOTH && l == g.L - 1;
  const double sweep_bytes = (double)n_interior(A.d) * ((A.ffi ? face_sweep_bytes(A, true)
                                                                : (A.hcoef ? 2.0 : (double)sizeof(T)) * popcount(A.mask)) +
                                                        4.0 * sizeof(T));
  SweepRun run;
  for (; q < c.pre(l); q++) {
    T* o = bufs[q & 1];
    if (cur) run.add(run_probe, s, sweep_bytes);
    smooth_probed<T>(l, A, lf, cur, b, o, (T)c.w(l, 0, q), c.cols, c.solo, s, l == c.top ? c.stage : STAGE_REGS);
    cur = o;
  }
  run.close();
  Level& C = g.lev[l - 1];
  T** xc = xbuf<T>(C);
  const double slot_bytes = A.hcoef ? 2.0 : (double)sizeof(T), nf = (double)n_interior(L.d);
  {
    // the slots, x, b and the restriction weights read; the coarse right-hand
    // side and the cleared coarse x written
    const bool face_rr = A.ffi && !g.si && !g.sj && !g.sk;  // the face form's restriction (tiled form only)
    Probed pr(VFS_PROBE_ALL, s, "k_resrestrict", l,
              nf * ((face_rr ? (A.ffc ? 40.0 : 24.0) : slot_bytes * popcount(A.mask)) + 3.0 * sizeof(T)) +
                  2.0 * n_interior(C.d) * sizeof(T));
    dbg("residual_restrict", l,
        launch_residual_restrict<T>(A, cur, b, rw_sel<T>(L, half), C.d, C.nvert, g.si, g.sj, g.sk, bbuf<T>(C), xc[0],
                                    s),
        s);
  }
  T* ec = vcycle<T>(g, l - 1, bbuf<T>(C), xc[0], xc[1], c, skip, s);
  {
    // code byte and coarse correction read, fine x written (read too when added)
    Probed pr(VFS_PROBE_ALL, s, "k_prolong", l,
              nf * (1.0 + (cur ? 2.0 : 1.0) * sizeof(T)) + (double)n_interior(C.d) * sizeof(T));
    if (!cur) {
      cur = bufs[q & 1];
      q++;
      dbg("prolong", l, launch_prolong<T>(L.d, L.pcode, C.d, ec, cur, 0, skip, s), s);
    } else {
      dbg("prolong_add", l, launch_prolong<T>(L.d, L.pcode, C.d, ec, cur, 1, skip, s), s);
    }
  }
  for (int r = 0; r < c.post(l); r++, q++) {
    T* o = bufs[q & 1];
    run.add(run_probe, s, sweep_bytes);
    smooth_probed<T>(l, A, lf, cur, b, o, (T)c.w(l, 1, r), c.cols, c.solo, s, l == c.top ? c.stage : STAGE_REGS);
    cur = o;
  }
  run.close();
  return cur;
}

// Damping of n sweeps: omega each (Jacobi), or 1 / theta_k at the roots
// theta_k = (hi + lo) / 2 + (hi - lo) / 2 cos((2k - 1) pi / (2n)), k = 1..n,
// of the degree-n Chebyshev polynomial on [lo, hi] (descending theta, so the
// smallest damping comes first); post-sweeps take them in reverse order.
void sweep_damping(const vfs_solve_params& p, int n, double* pre, double* post) {
  for (int k = 0; k < n; k++) {
    double w = p.omega;
    if (p.smoother == VFS_SMOOTH_CHEBYSHEV) {
      const double hi = p.cheb_hi, lo = p.cheb_hi / p.cheb_ratio;
      const double th = 0.5 * (hi + lo) + 0.5 * (hi - lo) * std::cos(M_PI * (2 * k + 1) / (2.0 * n));
      w = 1.0 / th;
    }
    pre[k] = w;
    post[n - 1 - k] = w;
  }
}

MGCfg mgcfg(const vfs_solve_params& p, int top, bool half_ok = true) {
  MGCfg c;
  c.nu1 = p.nu1;
  c.nu2 = p.nu2;
  c.ncoarse = 32;
  c.omega = p.omega;
  c.omega_c = p.omega;
  c.cols = p.smooth_cols;
  c.nu1c = p.nu1_coarse >= 0 ? p.nu1_coarse : p.nu1;
  c.nu2c = p.nu2_coarse >= 0 ? p.nu2_coarse : p.nu2;
  double tmp[MAXSWEEP];
  sweep_damping(p, c.nu1, c.wf[0], tmp);
  sweep_damping(p, c.nu2, tmp, c.wf[1]);
  sweep_damping(p, c.nu1c, c.wc[0], tmp);
  sweep_damping(p, c.nu2c, tmp, c.wc[1]);
  c.top = top;
  c.half = p.precision == VFS_MIXED && p.mg_half == 1 && half_ok;
  c.face = p.precision == VFS_MIXED && p.mg_half == 0;
  c.solo = false;
  c.stage = p.mg_stage;
  return c;
}

// z = M^{-1} v on the finest level (v FP64, z in T), optional skip flag.
// with_input == false: the finest-level input buffer already holds T(v).
template <typename T>
int precond(vfs_ctx* ctx, Grid& g, const vfs_solve_params& p, const double* v, T* z, T* tmp, const int* skip,
            cudaStream_t s, bool with_input = true, bool solo = false) {
  Level& F = g.lev[g.L - 1];
  T* bf = bbuf<T>(F);
  MGCfg mc = mgcfg(p, g.L - 1, g.half_ok);
  mc.solo = solo;
  const float* dinv = dinv_sel<T>(F, mc.half);
  if (with_input) dbg("scale_in", g.L - 1, launch_scale_in<T>(F.d, nullptr, v, bf, skip, s, dinv), s);
  T* res = vcycle<T>(g, g.L - 1, bf, z, tmp, mc, skip, s);
  if (res != z) CK(cudaMemcpyAsync(z, res, F.N * sizeof(T), cudaMemcpyDeviceToDevice, s));
  return VFS_OK;
}

// The outer operator is the aj-scaled FP64 operator (the multigrid path's
// form of the same system).
int apply_outer(Grid& g, const double* x, const double* b, double* y, const int* skip, cudaStream_t s) {
  Level& F = g.lev[g.L - 1];
  OpView<double> A{F.d, F.mcoef, F.mask, skip};
  return launch_apply64(A, x, b, y, s);
}

// ---------------------------------------------------------------------------
// Flexible GMRES(m), FP64 outer, preconditioned by one V-cycle in T.
// ---------------------------------------------------------------------------
struct Fgmres {
  // issue-side bookkeeping of one solve, so that several grids can be
  // interleaved (batched) by the same driver
  Grid* g;
  const vfs_solve_params* p;
  int it = 0, j = 0;
  int epoch = 0;  // the round's epoch (status copies of other rounds are ignored)
  bool observed = false, finished = false;
};

template <typename T>
T* zbase(Grid& g);
template <>
float* zbase<float>(Grid& g) { return g.Z32; }
template <>
double* zbase<double>(Grid& g) { return g.Z64; }

// Opening of a cycle: v0 = r / beta and the preconditioner input T(v0)
// (divided by D for the FP16 normalised multigrid operator).
template <typename T>
void fg_open_cycle(Grid& g, const vfs_solve_params& p, cudaStream_t s) {
  const size_t N = ncell(g.d);
  Level& F = g.lev[g.L - 1];
  dbg("v0", 0, launch_vec_scale_first(g.st, g.V, g.V, N, s), s);
  dbg("scale_in", 0,
      launch_scale_in<T>(F.d, nullptr, g.V, bbuf<T>(F), &g.st->done, s, dinv_sel<T>(F, mgcfg(p, g.L - 1, g.half_ok).half)), s);
}

template <typename T>
int fg_start(vfs_ctx* ctx, Fgmres& f, double atol, bool warm) {
  Grid& g = *f.g;
  const vfs_solve_params& p = *f.p;
  const size_t N = ncell(g.d);
  cudaStream_t s = g.s;
  KrylovState h{};
  h.m = p.restart;
  h.rtol = p.rtol;
  h.atol = atol;
  double* a = g.starr;
  h.H = a; a += (size_t)(p.restart + 1) * p.restart;
  h.cs = a; a += p.restart + 2;
  h.sn = a; a += p.restart + 2;
  h.g = a; a += p.restart + 2;
  h.y = a; a += p.restart + 2;
  h.h = a; a += p.restart + 2;
  h.hacc = a; a += p.restart + 2;
  h.vs = a;
  h.orth2 = p.orth == VFS_ORTH_CGS2;
  h.epoch = ++g.epoch;
  f.epoch = h.epoch;
  if (!g.st) {
    int r = galloc(ctx, g, (unsigned char**)&g.st, sizeof(KrylovState));
    if (r) return r;
  }
  CK(cudaMemcpyAsync(g.st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  if (!warm) CK(cudaMemsetAsync(g.phi, 0, N * sizeof(double), s));
  Level& F = g.lev[g.L - 1];
  dbg("scale_rhs", 0, launch_scale_in<double>(F.d, F.M + F.N * MP_AJ, g.b, g.bs, nullptr, s), s);
  dbg("bnorm", 0, launch_norm_init(g.st, g.bs, N, g.parts, 1, s), s);
  // r0 = aj b - A phi; from a cold start phi = 0 and r0 = aj b exactly
  if (warm) dbg("residual0", 0, apply_outer(g, g.phi, g.bs, g.V, &g.st->done, s), s);
  else CK(cudaMemcpyAsync(g.V, g.bs, N * sizeof(double), cudaMemcpyDeviceToDevice, s));
  dbg("beta", 0, launch_norm_init(g.st, g.V, N, g.parts, 0, s), s);
  fg_open_cycle<T>(g, p, s);
  g.hstat[0] = 0;
  f.it = 0;
  f.j = 0;
  f.observed = f.finished = false;
  return VFS_OK;
}

// One Arnoldi iteration as a fixed launch sequence (column index, basis
// slots and Krylov scalars all come from the device state), so it can be
// captured in a CUDA graph and replayed: V-cycle on T(v_j), w = A z_j with z
// stored to Z[j], CGS2, Hessenberg/Givens update, v_{j+1} and T(v_{j+1}),
// and a copy of the convergence flag to pinned memory (monotonic 0 -> 1).
// nv: the host's count of basis columns (column j + 1), for the probe's
// byte counts only (-1 when unknown, e.g. while capturing).
template <typename T>
void issue_krylov(Grid& g, const vfs_solve_params& p, cudaStream_t s, int nv = -1);

template <typename T>
void issue_iteration(Grid& g, const vfs_solve_params& p, cudaStream_t s, int nv = -1) {
  Level& F = g.lev[g.L - 1];
  MGCfg mc = mgcfg(p, g.L - 1, g.half_ok);
  mc.solo = g.solo;
  vcycle<T>(g, g.L - 1, bbuf<T>(F), xbuf<T>(F)[0], xbuf<T>(F)[1], mc, &g.st->done, s);
  issue_krylov<T>(g, p, s, nv);
}

// The iteration after its V-cycle (whose result is in the finest level's
// first buffer): w = A z, Gram-Schmidt, Arnoldi close, status copy.
template <typename T>
void issue_krylov(Grid& g, const vfs_solve_params& p, cudaStream_t s, int nv) {
  const size_t N = ncell(g.d);
  const double nvb = nv > 0 ? nv : 1, Nd = (double)N;
  const int* skip = &g.st->done;
  Level& F = g.lev[g.L - 1];
  T* zt = xbuf<T>(F)[0];
  const float* dinv = dinv_sel<T>(F, mgcfg(p, g.L - 1, g.half_ok).half);
  {
    // the FP64 slots, z read; w and the Z column written
    Probed pr(VFS_PROBE_APPLY64, s, "k_apply64_krylov", g.L - 1,
              (double)n_interior(F.d) * (8.0 * popcount(F.mask) + 2 * sizeof(T) + 8.0));
    OpView<double> A{F.d, F.mcoef, F.mask, skip};
    launch_apply64_krylov<T>(A, zt, zbase<T>(g), g.st, g.w, s);
  }
  dbg("apply64", g.L - 1, 0, s);
  {
    // the nv basis columns and w read (the finish reads block partials only)
    Probed pr(VFS_PROBE_ALL, s, "k_multidot", g.L - 1, Nd * (nvb + 1.0) * 8.0);
    dbg("multidot1", 0, launch_multidot(g.st, g.V, -1, g.w, N, g.parts, 1, s), s);
  }
  if (p.orth == VFS_ORTH_CGS) {
    // one pass: update, next column, next preconditioner input, norm partials
    {
      // w and the nv columns read; the new column and the multigrid input written
      Probed pr(VFS_PROBE_ALL, s, "k_cgs_update", g.L - 1,
                Nd * ((nvb + 2.0) * 8.0 + sizeof(T) + (dinv ? 4.0 : 0.0)));
      dbg("cgs_update", 0, launch_cgs_update<T>(g.st, g.V, g.w, bbuf<T>(F), N, g.parts, s, dinv), s);
    }
    {
      Probed pr(VFS_PROBE_ALL, s, "k_arnoldi_finish", g.L - 1, 0.);
      dbg("arnoldi", 0, launch_arnoldi_finish(g.st, krylov_nblocks(N), g.parts, s), s);
    }
    launch_status_copy(g.st, g.hstat, s);
    return;
  }
  {
    Probed pr(VFS_PROBE_ALL, s, "k_gs_update_dots", g.L - 1, Nd * (nvb + 2.0) * 8.0);
    if (g.m + 1 <= 32) {
      dbg("gs_update_dots", 0, launch_gs_update_dots(g.st, g.V, -1, g.w, N, g.parts, s, g.m + 1), s);
    } else {
      launch_gs_update(g.st, g.V, -1, g.w, N, g.parts, 1, s);
      launch_multidot(g.st, g.V, -1, g.w, N, g.parts, 2, s);
    }
  }
  {
    Probed pr(VFS_PROBE_ALL, s, "k_gs_update", g.L - 1, Nd * (nvb + 2.0) * 8.0);
    dbg("gs_update2", 0, launch_gs_update(g.st, g.V, -1, g.w, N, g.parts, 2, s), s);
  }
  {
    Probed pr(VFS_PROBE_ALL, s, "k_arnoldi_finish", g.L - 1, 0.);
    dbg("arnoldi", 0, launch_arnoldi_finish(g.st, krylov_nblocks(N), g.parts, s), s);
  }
  {
    Probed pr(VFS_PROBE_ALL, s, "k_vnext_in", g.L - 1, Nd * (16.0 + sizeof(T)));
    dbg("vnext_in", 0, launch_vnext_in<T>(g.st, g.w, nullptr, bbuf<T>(F), N, s, g.V, dinv), s);
  }
  launch_status_copy(g.st, g.hstat, s);
}

// The CGS2 sequence is graph-replayable up to 32 basis columns (the fused
// middle pass's largest capacity); the one-pass sequence for any restart.
bool graphs_allowed(const Grid& g, const vfs_solve_params& p) {
  return g_probe.kind == 0 && !g_debug && (p.orth == VFS_ORTH_CGS || g.m + 1 <= 32);
}

// The per-grid iteration graph (captured on first use; re-captured when the
// solve parameters change).
template <typename T>
int iteration_graph(vfs_ctx* ctx, Grid& g, const vfs_solve_params& p, cudaGraphExec_t* out) {
  const int prec = sizeof(T) == 4 ? VFS_MIXED : VFS_FP64;
  if (g.ig_exec && g.ig_prec == prec && g.ig_nu1 == p.nu1 && g.ig_nu2 == p.nu2 && g.ig_omega == p.omega &&
      g.ig_orth == p.orth && g.ig_cols == p.smooth_cols && g.ig_nu1c == p.nu1_coarse && g.ig_nu2c == p.nu2_coarse &&
      g.ig_half == p.mg_half && g.ig_solo == (int)g.solo && g.ig_smoother == p.smoother &&
      g.ig_cheb_hi == p.cheb_hi && g.ig_cheb_ratio == p.cheb_ratio && g.ig_stage == p.mg_stage) {
    *out = g.ig_exec;
    return VFS_OK;
  }
  if (g.ig_exec) {
    cudaGraphExecDestroy(g.ig_exec);
    g.ig_exec = nullptr;
  }
  cudaGraph_t graph = nullptr;
  const unsigned long long n0 = g_launches.load();
  CK(cudaStreamBeginCapture(g.s, cudaStreamCaptureModeThreadLocal));
  issue_iteration<T>(g, p, g.s);
  cudaError_t e = cudaStreamEndCapture(g.s, &graph);
  // captured launches run on replay, not now: count them per replay instead
  g.ig_kernels = g_launches.load() - n0;
  g_launches -= g.ig_kernels;
  if (e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return cuda_fail(ctx, e, "cudaStreamEndCapture");
  }
  e = cudaGraphInstantiate(&g.ig_exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
  g.ig_prec = prec;
  g.ig_nu1 = p.nu1;
  g.ig_nu2 = p.nu2;
  g.ig_omega = p.omega;
  g.ig_orth = p.orth;
  g.ig_cols = p.smooth_cols;
  g.ig_nu1c = p.nu1_coarse;
  g.ig_nu2c = p.nu2_coarse;
  g.ig_half = p.mg_half;
  g.ig_solo = (int)g.solo;
  g.ig_smoother = p.smoother;
  g.ig_cheb_hi = p.cheb_hi;
  g.ig_cheb_ratio = p.cheb_ratio;
  g.ig_stage = p.mg_stage;
  *out = g.ig_exec;
  return VFS_OK;
}

// Close a cycle (least squares, x update) and, unless finished, open the next
// one from the true residual of the updated phi.
template <typename T>
void fg_cycle_end(Grid& g, const vfs_solve_params& p, bool last, cudaStream_t s, int ncols = 0) {
  const size_t N = ncell(g.d);
  dbg("lsq", 0, launch_lsq_update(g.st, s), s);
  {
    // the cycle's ncols directions and phi read, phi written
    Probed pr(VFS_PROBE_ALL, s, "k_x_update", g.L - 1, (double)N * (ncols * (double)sizeof(T) + 16.0));
    dbg("x_update", 0, launch_x_update<T>(g.st, zbase<T>(g), N, g.phi, s), s);
  }
  dbg("restart_reset", 0, launch_restart_reset(g.st, s), s);
  if (last) return;
  {
    Level& F = g.lev[g.L - 1];
    Probed pr(VFS_PROBE_ALL, s, "k_apply64 (residual)", g.L - 1, (double)n_interior(F.d) * (8.0 * popcount(F.mask) + 24.0));
    apply_outer(g, g.phi, g.bs, g.V, &g.st->done, s);
  }
  launch_norm_init(g.st, g.V, N, g.parts, 0, s);
  fg_open_cycle<T>(g, p, s);
}

// Host bookkeeping after an iteration was issued on stream s: pipelined status
// check (the flag of the previous iteration) and the cycle end when due.
template <typename T>
int fg_after(vfs_ctx* ctx, Fgmres& f, cudaStream_t s) {
  Grid& g = *f.g;
  const vfs_solve_params& p = *f.p;
  f.it++;
  f.j++;
  CK(cudaEventRecord(g.ev[f.it & 1], s));
  // the flag of the previous iteration; while probing, of this one (no
  // iteration is issued past convergence, so the probe counts only work done)
  if (f.it >= 2 || g_probe.kind) {
    CK(cudaEventSynchronize(g.ev[(g_probe.kind ? f.it : f.it - 1) & 1]));
    if (g.hstat[0] && g.hstat[1] == f.epoch) f.observed = true;
  }
  if (f.observed || f.it >= p.maxit || f.j == p.restart) {
    const bool last = f.observed || f.it >= p.maxit;
    fg_cycle_end<T>(g, p, last, s, f.j);
    f.finished = last;
    f.j = 0;
  }
  return VFS_OK;
}

// Issue one iteration of one grid (graph replay when allowed) and do its
// bookkeeping.  Sets f.finished when done.
template <typename T>
int fg_step(vfs_ctx* ctx, Fgmres& f) {
  Grid& g = *f.g;
  if (graphs_allowed(g, *f.p)) {
    cudaGraphExec_t ex = nullptr;
    int r = iteration_graph<T>(ctx, g, *f.p, &ex);
    if (r) return r;
    CK(cudaGraphLaunch(ex, g.s));
    g_launches += g.ig_kernels;
  } else {
    issue_iteration<T>(g, *f.p, g.s, f.j + 1);
  }
  return fg_after<T>(ctx, f, g.s);
}

double initial_atol(const Grid& g, const vfs_solve_params& p) {
  if (p.div_tol <= 0.) return 0.;
  const double rmax_tol = p.div_tol * g.coeff / (g.dt * g.st_);
  // max |r| is typically 1/20 .. 1/200 of ||r||_2 / sqrt(n); start optimistic
  return rmax_tol * std::sqrt(std::max(g.nfluid, 1.)) * 0.05;
}

int check_params(vfs_ctx* ctx, const vfs_solve_params* p) {
  if (!p) return fail(ctx, VFS_ERR_ARG, "null solve params");
  if (p->restart < 1 || p->restart > MAXRESTART) return fail(ctx, VFS_ERR_ARG, "restart must be in [1, 64]");
  if (p->maxit < 1) return fail(ctx, VFS_ERR_ARG, "maxit must be >= 1");
  if (p->nu1 < 0 || p->nu2 < 0 || p->nu1 + p->nu2 < 1) return fail(ctx, VFS_ERR_ARG, "need at least one smoothing sweep");
  {
    const int a = p->nu1_coarse >= 0 ? p->nu1_coarse : p->nu1, b = p->nu2_coarse >= 0 ? p->nu2_coarse : p->nu2;
    if (p->nu1_coarse < -1 || p->nu2_coarse < -1 || a + b < 1)
      return fail(ctx, VFS_ERR_ARG, "nu1_coarse / nu2_coarse: -1 (as nu1 / nu2) or >= 0, at least one sweep");
  }
  if (!(p->rtol > 0.)) return fail(ctx, VFS_ERR_ARG, "rtol must be > 0");
  if (!(p->omega > 0. && p->omega < 2.)) return fail(ctx, VFS_ERR_ARG, "omega must be in (0, 2)");
  if (!(p->div_tol >= 0.)) return fail(ctx, VFS_ERR_ARG, "div_tol must be >= 0");
  if (p->precision != VFS_FP64 && p->precision != VFS_MIXED) return fail(ctx, VFS_ERR_ARG, "unknown precision");
  if (p->proj_exact != 0 && p->proj_exact != 1) return fail(ctx, VFS_ERR_ARG, "proj_exact must be 0 or 1");
  if (p->mg_grouped != 0 && p->mg_grouped != 1) return fail(ctx, VFS_ERR_ARG, "mg_grouped must be 0 or 1");
  if (p->mg_stage != STAGE_REGS && p->mg_stage != STAGE_TMA) return fail(ctx, VFS_ERR_ARG, "mg_stage must be 0 or 1");
  if (p->orth != VFS_ORTH_CGS && p->orth != VFS_ORTH_CGS2)
    return fail(ctx, VFS_ERR_ARG, "orth must be VFS_ORTH_CGS or VFS_ORTH_CGS2");
  if (p->smooth_cols != 0 && p->smooth_cols != 8 && p->smooth_cols != 16 && p->smooth_cols != 32)
    return fail(ctx, VFS_ERR_ARG, "smooth_cols must be 0 (automatic), 8, 16 or 32");
  if (p->mg_half < 0 || p->mg_half > 2) return fail(ctx, VFS_ERR_ARG, "mg_half must be 0, 1 or 2");
  if (p->nu1 > MAXSWEEP || p->nu2 > MAXSWEEP || p->nu1_coarse > MAXSWEEP || p->nu2_coarse > MAXSWEEP)
    return fail(ctx, VFS_ERR_ARG, "at most 64 smoothing sweeps per level and side");
  if (p->smoother != VFS_SMOOTH_JACOBI && p->smoother != VFS_SMOOTH_CHEBYSHEV)
    return fail(ctx, VFS_ERR_ARG, "smoother must be VFS_SMOOTH_JACOBI or VFS_SMOOTH_CHEBYSHEV");
  if (p->smoother == VFS_SMOOTH_CHEBYSHEV && !(p->cheb_hi > 0. && p->cheb_hi <= 4. && p->cheb_ratio > 1.))
    return fail(ctx, VFS_ERR_ARG, "Chebyshev smoother: cheb_hi must be in (0, 4] and cheb_ratio > 1");
  return VFS_OK;
}

// ---------------------------------------------------------------------------
// Solve jobs.  One solve (optionally with the step's flux balance and RHS
// before it and pressure update, projection, Contra2Cart and divergence
// after it) is a state machine whose waits are events the driver polls, so
// that many grids' solves can be in flight together:
//   START  inputs, step_pre, FGMRES start
//   ITER   Arnoldi iterations (graph replays) until the device flag or maxit
//   CHECK  true aj-scaled residual ||r|| and the exact masked max |r| (the
//          divergence the projection will leave, times coeff / (dt st)) are
//          on their way to pinned memory; when they arrive, either the solve
//          closes or, while max |r| is above div_tol, another FGMRES round
//          starts from the current phi with a tighter L2 target (at most 8)
//   POST   null-space removal, phi finish, step_post and the outputs are on
//          their way; when they arrive the job is DONE.
// A job's work is ordered on its grid's stream; its host transfers run on
// the grid's copy stream, joined to the step stream by events.
// ---------------------------------------------------------------------------
enum JobPhase { J_START = 0, J_ITER, J_CHECK, J_POST, J_DONE };

void step_pre(Grid& g, double dt, double st, double coeff);
// Slabs of the flux upload and download: one per 4 MiB of AoS fluxes, 1 to 8.
int transfer_slabs(size_t ncells) {
  const size_t b = 3 * ncells * sizeof(double);
  return (int)std::max<size_t>(1, std::min<size_t>(8, b >> 22));
}

int step_post(Grid& g, double dt, double st, double coeff, bool exact, double* u_out = nullptr,
              double* p_out = nullptr, bool p_in_pending = false);

struct Job {
  Grid* g = nullptr;
  vfs_solve_params p{};   // the caller's parameters
  vfs_solve_params pr{};  // this round's (maxit shrinks over the rounds)
  Fgmres f{};
  bool pre = false, post = false;
  const double* u_in = nullptr;  // host AoS U* (with pre); else the resident U*
  const double* p_in = nullptr;  // host pressure (with pre), else the resident one
  double* u_out = nullptr;       // host AoS corrected fluxes (with post)
  double* p_out = nullptr;       // host pressure (with post)
  double dt = 0.04, st = 1., coeff = 1.;
  int phase = J_START, round = 0, iters = 0, refine = 0;
  double atol = 0., rmax_tol = 0., prev_rmax = 0.;
  double bnorm0 = 0.;  // ||aj b|| of the step's first pass (the rtol reference of later passes)
  vfs_solve_info info{};
  double divmax = 0.;
  int rc = VFS_OK;
  std::string err;
  bool pending = false;  // batch: work on the grid's stream since the last tick
  bool p_in_pending = false;  // the pressure upload is on the copy stream
  long long ticket = 0;
  bool mixed() const { return p.precision == VFS_MIXED; }
};

}  // namespace

struct vfs_job_box {
  Job job;
};

namespace {

int job_fail(vfs_ctx* ctx, Job& J, int rc) {
  J.rc = rc;
  J.err = ctx->err;
  J.phase = J_DONE;
  return rc;
}

template <typename T>
int job_start(vfs_ctx* ctx, Job& J) {
  Grid& g = *J.g;
  int r = ensure_mg<T>(ctx, g);
  if (!r) r = ensure_krylov(ctx, g, J.p.restart, J.p.precision);
  if (r) return job_fail(ctx, J, r);
  const size_t N = ncell(g.d);
  CK(cudaEventRecord(g.t0, g.s));
  if (J.pre) {
    if (J.u_in || J.p_in) {
      // host uploads run on the copy stream, after the step stream's earlier
      // work on the staging buffer, the fluxes and the pressure
      CK(cudaEventRecord(g.ev_uin, g.s));
      CK(cudaStreamWaitEvent(g.cs, g.ev_uin, 0));
    }
    if (J.u_in) {
      // the fluxes go up in k-plane slabs on the copy stream, each slab
      // converted to SoA on the step stream while the next one is in flight
      const int mz = g.d.mz;
      const size_t P = (size_t)g.d.mx * g.d.my;
      const int S = std::min(mz, transfer_slabs(N));
      for (int q = 0; q < S; q++) {
        const size_t c0 = (size_t)(mz * (long long)q / S) * P, c1 = (size_t)(mz * (long long)(q + 1) / S) * P;
        CK(cudaMemcpyAsync(g.aos + 3 * c0, J.u_in + 3 * c0, 3 * (c1 - c0) * sizeof(double), cudaMemcpyHostToDevice,
                           g.cs));
        CK(cudaEventRecord(g.ev_uin, g.cs));
        CK(cudaStreamWaitEvent(g.s, g.ev_uin, 0));
        launch_aos2soa(c1 - c0, g.aos + 3 * c0, g.u + c0, g.u + N + c0, g.u + 2 * N + c0, g.s);
      }
    } else {
      CK(cudaMemcpyAsync(g.u, g.ustar, 3 * N * sizeof(double), cudaMemcpyDeviceToDevice, g.s));
    }
    if (J.p_in) {  // needed only at the pressure update: upload during the solve,
                   // on the copy stream after the fluxes
      CK(cudaMemcpyAsync(g.p, J.p_in, N * sizeof(double), cudaMemcpyHostToDevice, g.cs));
      CK(cudaEventRecord(g.ev_pin, g.cs));
      J.p_in_pending = true;
    }
    step_pre(g, J.dt, J.st, J.coeff);
  }
  J.rmax_tol = J.p.div_tol > 0. ? J.p.div_tol * g.coeff / (g.dt * g.st_) : 0.;
  J.prev_rmax = 0.;
  J.atol = initial_atol(g, J.p);
  J.pr = J.p;
  J.f = Fgmres{&g, &J.pr};
  r = fg_start<T>(ctx, J.f, J.atol, J.p.warm_start != 0);
  if (r) return job_fail(ctx, J, r);
  J.phase = J_ITER;
  J.pending = true;
  return VFS_OK;
}

// After the FGMRES round ended: the true residual and its exact masked max
// on their way to pinned memory.
int job_check_enqueue(vfs_ctx* ctx, Job& J) {
  Grid& g = *J.g;
  const size_t N = ncell(g.d);
  cudaStream_t s = g.s;
  Level& F = g.lev[g.L - 1];
  {
    Probed pr(VFS_PROBE_ALL, s, "k_apply64 (residual)", g.L - 1, (double)n_interior(F.d) * (8.0 * popcount(F.mask) + 24.0));
    dbg("true_residual", 0, apply_outer(g, g.phi, g.bs, g.w, nullptr, s), s);
  }
  {
    Probed pr(VFS_PROBE_ALL, s, "k_norm2 + k_masked_absmax", g.L - 1, (double)N * (8.0 + 8.0 + (g.nb8 ? 1.0 : 8.0)));
    dbg("norm2", 0, launch_norm2(g.w, N, g.parts, g.scal + 16, s), s);
    dbg("masked_max", 0, launch_masked_absmax(F.d, g.w, F.nvert, g.parts, g.scal + 17, s, g.nb8), s);
  }
  CK(cudaMemcpyAsync(g.hk, g.st, sizeof(KrylovState), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(g.hv, g.scal + 16, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(g.ev_chk, s));
  J.phase = J_CHECK;
  J.pending = true;
  return VFS_OK;
}

// The check arrived: close the solve or start another round.
template <typename T>
int job_check_eval(vfs_ctx* ctx, Job& J) {
  Grid& g = *J.g;
  const KrylovState h = *g.hk;
  const double rn = g.hv[0], rmax = g.hv[1];
  if (!(h.bnorm == h.bnorm) || !(h.resid == h.resid) || !(rn == rn)) {
    fail(ctx, VFS_ERR_NUMERIC, "NaN in the solve");
    return job_fail(ctx, J, VFS_ERR_NUMERIC);
  }
  J.iters += h.it;
  // a further projection pass solves for the divergence the earlier passes
  // left; its residual is that of the whole step, measured against the first
  // pass's right-hand side
  const double bref = J.refine ? J.bnorm0 : h.bnorm;
  const bool rel_ok = rn <= J.p.rtol * bref * 1.0000001 || bref == 0.;
  const bool div_ok = J.p.div_tol <= 0. || rmax <= J.rmax_tol;
  // a finish round that no longer halves the masked max has met the FP64
  // rounding floor of this grid: the divergence target is out of reach
  const bool floor = !div_ok && J.round > 0 && rmax > 0.5 * J.prev_rmax;
  J.prev_rmax = rmax;
  if ((rel_ok && (div_ok || floor)) || J.iters >= J.p.maxit || h.bnorm == 0. || J.round == 7) {
    if (!J.refine) J.bnorm0 = h.bnorm;
    cudaStream_t s = g.s;
    Level& F = g.lev[g.L - 1];
    const size_t N = ncell(g.d);
    {
      // per region: nvert and phi read; nvert and phi read, phi written
      Probed pr(VFS_PROBE_ALL, s, "k_fluid_sum + k_sub_mean", g.L - 1, (double)N * 40.0 * g.ncomp);
      dbg("remove_mean", 0, launch_remove_mean(F.d, F.nvert, g.phi, g.parts, g.scal, s, g.comp, g.ncomp), s);
    }
    {
      Probed pr(VFS_PROBE_ALL, s, "k_phi_zero + ghosts", g.L - 1, (double)N * 16.0);
      dbg("phi_finish", 0, launch_phi_finish(F.d, F.nvert, g.phi, s), s);
    }
    CK(cudaEventRecord(g.t1, s));
    if (J.post) {
      const int rp = step_post(g, J.dt, J.st, J.coeff, J.p.proj_exact != 0, J.u_out, J.p_out, J.p_in_pending);
      J.p_in_pending = false;
      if (rp) return job_fail(ctx, J, cuda_fail(ctx, (cudaError_t)rp, "step outputs"));
      CK(cudaMemcpyAsync(g.hv + 2, g.scal + 8, sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    CK(cudaEventRecord(g.ev_done, s));
    J.info.iterations = J.iters;
    J.info.converged = rel_ok && (div_ok || floor);
    J.info.div_limited = (!div_ok && floor) ? 1 : 0;
    J.info.mg_half_used = mgcfg(J.p, g.L - 1, g.half_ok).half ? 1 : 0;
    J.info.bnorm = bref;
    J.info.relres = bref > 0. ? rn / bref : 0.;
    J.phase = J_POST;
    J.pending = true;
    return VFS_OK;
  }
  J.atol = std::min(J.atol > 0. ? J.atol : rn, rn) * (div_ok ? 1. : 0.5 * J.rmax_tol / rmax);
  J.pr.maxit = J.p.maxit - J.iters;
  J.round++;
  const int r = fg_start<T>(ctx, J.f, J.atol, true);
  if (r) return job_fail(ctx, J, r);
  J.phase = J_ITER;
  J.pending = true;
  return VFS_OK;
}

// The step's outputs arrived.  The residual test bounds the divergence the
// projection leaves up to the rounding of the flux update and of phi itself:
// where |phi| is large (strong stretching, N(0, 1) fluxes: |phi| ~ 1e3) the
// FP64 phi cannot carry differences fine enough for div_tol, and the solve
// rounds stop at that floor.  When the measured max |div u| still exceeds
// div_tol, one more projection pass on the corrected fluxes removes the rest:
// RHS of the corrected U, a solve from zero (its phi is small, so its floor
// is far lower), pressure update and projection (the pressure accumulates
// both passes, as one tighter solve would).  At most two further passes.
template <typename T>
int job_post_eval(vfs_ctx* ctx, Job& J) {
  Grid& g = *J.g;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, g.t0, g.t1);
  J.info.time_ms = ms;
  if (J.post) J.divmax = g.hv[2];
  if (J.post && J.p.div_tol > 0. && J.divmax > J.p.div_tol && J.refine < 2 && J.iters < J.p.maxit) {
    J.refine++;
    step_pre(g, J.dt, J.st, J.coeff);
    J.round = 0;
    J.prev_rmax = 0.;
    J.pr.maxit = J.p.maxit - J.iters;
    // the pass stops on the divergence target (its rtol reference is the
    // first pass's right-hand side, checked on the host)
    J.pr.rtol = 1.;
    J.atol = initial_atol(g, J.p);
    const int r = fg_start<T>(ctx, J.f, J.atol, false);
    if (r) return job_fail(ctx, J, r);
    J.phase = J_ITER;
    J.pending = true;
    return VFS_OK;
  }
  // with the step's divergence measured, div_limited reports the outcome
  if (J.post && J.p.div_tol > 0.) J.info.div_limited = J.divmax > J.p.div_tol ? 1 : 0;
  // a bounded wait of the tensor-copy sweep that ran out leaves garbage
  if (J.p.mg_stage == STAGE_TMA && smooth_tma_take_error())
    return job_fail(ctx, J, fail(ctx, VFS_ERR_CUDA, "tensor-copy sweep: a bounded wait ran out"));
  J.phase = J_DONE;
  return VFS_OK;
}

// Advance one job on its own stream as far as it goes without waiting
// (an iteration's bookkeeping waits for the previous iteration of the same
// grid only).  Returns 1 if the job moved, 0 if it waits on the device.
template <typename T>
int job_advance(vfs_ctx* ctx, Job& J) {
  Grid& g = *J.g;
  switch (J.phase) {
    case J_START:
      job_start<T>(ctx, J);
      return 1;
    case J_ITER: {
      const int r = fg_step<T>(ctx, J.f);
      if (r) return job_fail(ctx, J, r), 1;
      if (J.f.finished) job_check_enqueue(ctx, J);
      return 1;
    }
    case J_CHECK: {
      const cudaError_t e = cudaEventQuery(g.ev_chk);
      if (e == cudaErrorNotReady) return 0;
      if (e != cudaSuccess) return job_fail(ctx, J, cuda_fail(ctx, e, "check")), 1;
      job_check_eval<T>(ctx, J);
      return 1;
    }
    case J_POST: {
      const cudaError_t e = cudaEventQuery(g.ev_done);
      if (e == cudaErrorNotReady) return 0;
      if (e != cudaSuccess) return job_fail(ctx, J, cuda_fail(ctx, e, "post")), 1;
      job_post_eval<T>(ctx, J);
      return 1;
    }
    default:
      return 0;
  }
}
int job_advance_any(vfs_ctx* ctx, Job& J) { return J.mixed() ? job_advance<float>(ctx, J) : job_advance<double>(ctx, J); }

// Block until one of the jobs' awaited events completes (no busy spin).
void wait_any(std::vector<Job*>& jobs) {
  for (Job* J : jobs) {
    if (J->phase == J_CHECK) { cudaEventSynchronize(J->g->ev_chk); return; }
    if (J->phase == J_POST) { cudaEventSynchronize(J->g->ev_done); return; }
  }
}

// Run jobs to completion, each on its grid's stream (single solves; the
// serving loop uses job_advance directly).
int run_jobs_streams(vfs_ctx* ctx, std::vector<Job*>& jobs) {
  for (Job* J : jobs) J->g->solo = jobs.size() == 1;
  for (;;) {
    int moved = 0, live = 0;
    for (Job* J : jobs) {
      if (J->phase == J_DONE) continue;
      moved += job_advance_any(ctx, *J);
      if (J->phase != J_DONE) live++;
    }
    if (!live) return VFS_OK;
    if (!moved) wait_any(jobs);
  }
}

// ---------------------------------------------------------------------------
// Batched iterations: ONE CUDA graph per tick holds the next Arnoldi iteration
// of every grid in the batch, each as its own branch (captured from the
// grid's stream, forked from and joined to the batch stream), so the
// iterations of all grids run concurrently from one launch.  Grids whose
// device flag is set skip their kernels; the graph is re-captured when a grid
// needs iterations and is not in it, or when fewer than half of its branches
// are still iterating.  Out-of-graph work of a grid (cycle ends, checks,
// restarts) stays on the grid's stream, ordered after the latest tick, and
// the next tick waits for it.
// ---------------------------------------------------------------------------
struct BatchGraph {
  cudaGraphExec_t exec = nullptr;
  std::vector<Job*> members;
  unsigned long long kernels = 0;
  std::vector<void*> tables;  // work-item tables of the grouped launches (every capture's, freed at the end)
  std::vector<cudaEvent_t> stage_done;  // end of each group's stages within a tick
  ~BatchGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    for (void* t : tables) cudaFree(t);
    for (cudaEvent_t e : stage_done) cudaEventDestroy(e);
  }
};

// ---------------------------------------------------------------------------
// Grouped V-cycles (mg_group.h): the V-cycle of each member whose solve
// allows it (mg_grouped = 1, full coarsening, not the FP16 operator) is
// recorded as an operation list that mirrors vcycle() (same buffers, same
// damping, same tiles); operation i of every list runs in stage i, one
// launch per kernel instantiation present in the stage, each with a table
// of one item per grid.  The tick graph runs the stages on the batch stream
// and then each member's Krylov part on its own stream.
// ---------------------------------------------------------------------------
enum GOpKind { GOP_SMOOTH, GOP_RESTRICT, GOP_PROLONG, GOP_PROLONG_ADD, GOP_GEMV };
template <typename T>
struct GOp {
  int kind, lev;
  const T* x;
  const T* b;
  T* y;
  T* y2;
  double w;
};

template <typename T>
T* group_ops(Grid& g, int l, T* b, T* xa, T* xb, const MGCfg& c, std::vector<GOp<T>>& ops) {
  Level& L = g.lev[l];
  const int W = level_writes(g, l, c);
  T* bufs[2] = {xa, xb};
  if (((W - 1) & 1) == 1) std::swap(bufs[0], bufs[1]);
  if (l == 0) {
    if (binv<T>(L)) {
      ops.push_back(GOp<T>{GOP_GEMV, 0, nullptr, b, bufs[0], nullptr, 0.});
      return bufs[0];
    }
    T* cur = nullptr;
    for (int q = 0; q < c.ncoarse; q++) {
      T* o = bufs[q & 1];
      ops.push_back(GOp<T>{GOP_SMOOTH, 0, cur, b, o, nullptr, c.omega_c});
      cur = o;
    }
    return cur;
  }
  int q = 0;
  T* cur = nullptr;
  for (; q < c.pre(l); q++) {
    T* o = bufs[q & 1];
    ops.push_back(GOp<T>{GOP_SMOOTH, l, cur, b, o, nullptr, c.w(l, 0, q)});
    cur = o;
  }
  Level& C = g.lev[l - 1];
  T** xc = xbuf<T>(C);
  ops.push_back(GOp<T>{GOP_RESTRICT, l, cur, b, bbuf<T>(C), xc[0], 0.});
  T* ec = group_ops<T>(g, l - 1, bbuf<T>(C), xc[0], xc[1], c, ops);
  if (!cur) {
    cur = bufs[q & 1];
    q++;
    ops.push_back(GOp<T>{GOP_PROLONG, l, ec, nullptr, cur, nullptr, 0.});
  } else {
    ops.push_back(GOp<T>{GOP_PROLONG_ADD, l, ec, nullptr, cur, nullptr, 0.});
  }
  for (int r = 0; r < c.post(l); r++, q++) {
    T* o = bufs[q & 1];
    ops.push_back(GOp<T>{GOP_SMOOTH, l, cur, b, o, nullptr, c.w(l, 1, r)});
    cur = o;
  }
  return cur;
}

// The item of one operation on one grid: its kernel, tiles and shared memory.
template <typename T>
void group_item(Grid& g, const GOp<T>& op, const MGCfg& c, const int* skip, int* kind, GroupItem<T>* it, int* blocks,
                size_t* smem) {
  Level& L = g.lev[op.lev];
  const bool face = sizeof(T) == 4 && c.face && face_level(L);
  const bool ch = face_level(L);  // the 11-slot set
  GroupItem<T> t{};
  t.A = mgview<T>(L, skip, false, face);
  t.skip = skip;
  t.x = op.x;
  t.b = op.b;
  t.y = op.y;
  t.y2 = op.y2;
  t.w = (T)op.w;
  *smem = 0;
  const int ni = L.d.mx - 2, nj = L.d.my - 2, nk = L.d.mz - 2;
  switch (op.kind) {
    case GOP_SMOOTH: {
      t.lf = lf_sel<T>(L, false);
      t.tw = smooth_tw<T>(ni, nj, nk, c.cols, VFS_SMOOTH_NARROW_SHARED != 0);  // grouped grids share the GPU
      t.gx = (ni + t.tw - 1) / t.tw;
      t.gy = nk;
      *blocks = t.gx * nk;
      *smem = smooth_smem<T>(t.tw, nj);
      const int zg = op.x ? 0 : 1;
      *kind = (face ? GK_SMOOTH_FACE : ch ? GK_SMOOTH_CH : GK_SMOOTH_ALL) + zg;
      break;
    }
    case GOP_RESTRICT: {
      Level& C = g.lev[op.lev - 1];
      t.rw = rw_sel<T>(L, false);
      t.c = C.d;
      t.nvc = C.nvert;
      t.gx = (C.d.mx - 2 + 31) / 32;
      t.gy = (C.d.my - 2 + 3) / 4;
      *blocks = t.gx * t.gy * (C.d.mz - 2);
      *kind = face ? GK_RESTRICT_FACE : ch ? GK_RESTRICT_CH : GK_RESTRICT_ALL;
      break;
    }
    case GOP_PROLONG:
    case GOP_PROLONG_ADD: {
      Level& C = g.lev[op.lev - 1];
      t.c = C.d;
      t.pcode = L.pcode;
      t.add = op.kind == GOP_PROLONG_ADD;
      t.gx = (ni + 31) / 32;
      t.gy = (nj + 7) / 8;
      *blocks = t.gx * t.gy * ((nk + 3) / 4);
      *kind = GK_PROLONG;
      break;
    }
    default: {  // GOP_GEMV
      t.Binv = binv<T>(L);
      t.n = L.nco;
      *blocks = (L.nco + 7) / 8;
      *smem = (size_t)L.nco * sizeof(T);
      *kind = GK_GEMV;
      break;
    }
  }
  *it = t;
}

struct GroupLaunch {
  int kind, nitems, nblocks;
  size_t off, smem;  // first item in the table, dynamic shared memory
};

// The stages of the grouped V-cycles of `jobs` (all of multigrid precision
// T): their launches and the item table (host side).
template <typename T>
void group_plan(std::vector<Job*>& jobs, std::vector<GroupLaunch>& launches, std::vector<GroupItem<T>>& table) {
  std::vector<std::vector<GOp<T>>> lists(jobs.size());
  std::vector<MGCfg> cfg(jobs.size());
  size_t stages = 0;
  for (size_t q = 0; q < jobs.size(); q++) {
    Grid& g = *jobs[q]->g;
    Level& F = g.lev[g.L - 1];
    cfg[q] = mgcfg(jobs[q]->p, g.L - 1, g.half_ok);
    group_ops<T>(g, g.L - 1, bbuf<T>(F), xbuf<T>(F)[0], xbuf<T>(F)[1], cfg[q], lists[q]);
    stages = std::max(stages, lists[q].size());
  }
  for (size_t i = 0; i < stages; i++) {
    std::vector<GroupItem<T>> bucket[GK_COUNT];
    int nb[GK_COUNT] = {0};
    size_t sm[GK_COUNT] = {0};
    for (size_t q = 0; q < jobs.size(); q++) {
      if (i >= lists[q].size()) continue;
      Grid& g = *jobs[q]->g;
      int kind = 0, blocks = 0;
      size_t smem = 0;
      GroupItem<T> it;
      group_item<T>(g, lists[q][i], cfg[q], &g.st->done, &kind, &it, &blocks, &smem);
      it.start = nb[kind];
      nb[kind] += blocks;
      sm[kind] = std::max(sm[kind], smem);
      bucket[kind].push_back(it);
    }
    for (int k = 0; k < GK_COUNT; k++) {
      if (bucket[k].empty()) continue;
      launches.push_back(GroupLaunch{k, (int)bucket[k].size(), nb[k], table.size(), sm[k]});
      table.insert(table.end(), bucket[k].begin(), bucket[k].end());
    }
  }
}

// Grids grouped together: the same multigrid precision, number of levels
// and interior cell count to within a factor of two (so that a stage's
// launches do not wait long on one grid's larger tiles).
std::string group_key(const Job& J) {
  const Grid& g = *J.g;
  const double cells = (double)n_interior(g.d);
  return std::to_string(J.mixed() ? 4 : 8) + ":" + std::to_string(g.L) + ":" +
         std::to_string((int)std::lround(std::log2(std::max(cells, 1.))));
}

// Members whose V-cycle may run grouped (the grouped kernels run the 11-slot
// face form only: a mixed grid with i-j or j-k cross terms on some level,
// whose own V-cycle uses the general face form there, runs ungrouped).
bool groupable(const Job& J) {
  const Grid& g = *J.g;
  const MGCfg c = mgcfg(J.p, g.L - 1, g.half_ok);
  if (J.p.mg_grouped == 0 || g.si || g.sj || g.sk || c.half) return false;
  if (J.mixed() && c.face)
    for (int l = 0; l < g.L; l++)
      if (!face_level(g.lev[l])) return false;
  return true;
}

// Uploads a grouped plan's table (a device buffer owned by bg) and returns
// its device address.
template <typename T>
int group_upload(vfs_ctx* ctx, cudaStream_t s0, const std::vector<GroupItem<T>>& table, BatchGraph& bg,
                 const GroupItem<T>** out) {
  *out = nullptr;
  if (table.empty()) return VFS_OK;
  void* d = nullptr;
  CK(cudaMalloc(&d, table.size() * sizeof(GroupItem<T>)));
  bg.tables.push_back(d);
  CK(cudaMemcpyAsync(d, table.data(), table.size() * sizeof(GroupItem<T>), cudaMemcpyHostToDevice, s0));
  CK(cudaStreamSynchronize(s0));  // the host table goes out of scope
  *out = (const GroupItem<T>*)d;
  return VFS_OK;
}

int batch_capture(vfs_ctx* ctx, cudaStream_t s0, cudaEvent_t fork, std::vector<cudaEvent_t>& joins,
                  std::vector<Job*>& members, BatchGraph& bg) {
  if (bg.exec) {
    cudaGraphExecDestroy(bg.exec);
    bg.exec = nullptr;
  }
  while (joins.size() < members.size()) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    joins.push_back(e);
  }
  // grouped V-cycles: groups, plans and tables before the capture
  std::map<std::string, std::vector<size_t>> groups;
  std::vector<char> grouped(members.size(), 0);
  for (size_t q = 0; q < members.size(); q++) {
    if (!groupable(*members[q])) continue;
    grouped[q] = 1;
    groups[group_key(*members[q])].push_back(q);
  }
  struct Plan {
    std::vector<size_t> idx;
    bool f32;
    std::vector<GroupLaunch> launches;
    const GroupItem<float>* d32 = nullptr;
    const GroupItem<double>* d64 = nullptr;
  };
  std::vector<Plan> plans;
  for (auto& kv : groups) {
    Plan P;
    P.idx = kv.second;
    std::vector<Job*> js;
    for (size_t q : P.idx) js.push_back(members[q]);
    P.f32 = js[0]->mixed();
    if (P.f32) {
      std::vector<GroupItem<float>> t;
      group_plan<float>(js, P.launches, t);
      if (int r = group_upload<float>(ctx, s0, t, bg, &P.d32)) return r;
    } else {
      std::vector<GroupItem<double>> t;
      group_plan<double>(js, P.launches, t);
      if (int r = group_upload<double>(ctx, s0, t, bg, &P.d64)) return r;
    }
    plans.push_back(std::move(P));
  }
  while (bg.stage_done.size() < plans.size()) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    bg.stage_done.push_back(e);
  }
  const unsigned long long n0 = g_launches.load();
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
  cudaEventRecord(fork, s0);
  // members not grouped: their whole iteration on their own streams
  for (size_t q = 0; q < members.size(); q++) {
    if (grouped[q]) continue;
    Grid& g = *members[q]->g;
    cudaStreamWaitEvent(g.s, fork, 0);
    if (members[q]->mixed()) issue_iteration<float>(g, members[q]->p, g.s);
    else issue_iteration<double>(g, members[q]->p, g.s);
    cudaEventRecord(joins[q], g.s);
  }
  // each group: its V-cycle stages on its first member's stream, then every
  // member's Krylov part on the member's own stream
  for (size_t k = 0; k < plans.size(); k++) {
    const Plan& P = plans[k];
    cudaStream_t gs = members[P.idx[0]]->g->s;
    cudaStreamWaitEvent(gs, fork, 0);
    for (const GroupLaunch& gl : P.launches) {
      if (P.f32) launch_group<float>(gl.kind, P.d32 + gl.off, gl.nitems, gl.nblocks, gl.smem, gs);
      else launch_group<double>(gl.kind, P.d64 + gl.off, gl.nitems, gl.nblocks, gl.smem, gs);
    }
    cudaEventRecord(bg.stage_done[k], gs);
    for (size_t q : P.idx) {
      Grid& g = *members[q]->g;
      cudaStreamWaitEvent(g.s, bg.stage_done[k], 0);
      if (members[q]->mixed()) issue_krylov<float>(g, members[q]->p, g.s);
      else issue_krylov<double>(g, members[q]->p, g.s);
      cudaEventRecord(joins[q], g.s);
    }
  }
  for (size_t q = 0; q < members.size(); q++) cudaStreamWaitEvent(s0, joins[q], 0);
  cudaError_t e = cudaStreamEndCapture(s0, &graph);
  bg.kernels = g_launches.load() - n0;
  g_launches -= bg.kernels;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batch capture");
  e = cudaGraphInstantiate(&bg.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batch graph instantiate");
  bg.members = members;
  return VFS_OK;
}

template <typename T>
int batch_after_tick(vfs_ctx* ctx, Job& J, cudaEvent_t tick, bool have_prev) {
  Grid& g = *J.g;
  Fgmres& f = J.f;
  f.it++;
  f.j++;
  if (have_prev && g.hstat[0] && g.hstat[1] == f.epoch) f.observed = true;
  if (f.observed || f.it >= f.p->maxit || f.j == f.p->restart) {
    const bool last = f.observed || f.it >= f.p->maxit;
    CK(cudaStreamWaitEvent(g.s, tick, 0));
    fg_cycle_end<T>(g, *f.p, last, g.s);
    J.pending = true;
    f.finished = last;
    f.j = 0;
    if (last) return job_check_enqueue(ctx, J);
  }
  return VFS_OK;
}

int run_jobs_batch(vfs_ctx* ctx, std::vector<Job*>& jobs, cudaStream_t s0) {
  for (Job* J : jobs) J->g->solo = false;
  cudaEvent_t fork = nullptr, ticks[2] = {nullptr, nullptr};
  std::vector<cudaEvent_t> joins;
  BatchGraph bg;
  auto cleanup = [&]() {
    if (fork) cudaEventDestroy(fork);
    for (cudaEvent_t e : ticks) if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : joins) cudaEventDestroy(e);
  };
  struct Guard {
    std::function<void()> f;
    ~Guard() { f(); }
  } guard{cleanup};
  CK(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ticks[0], cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ticks[1], cudaEventDisableTiming));
  for (Job* J : jobs) {
    if (J->mixed()) job_start<float>(ctx, *J);
    else job_start<double>(ctx, *J);
  }
  long long t = 0;
  bool ticked_prev = false;
  for (;;) {
    std::vector<Job*> iter;
    int live = 0;
    for (Job* J : jobs) {
      if (J->phase == J_DONE) continue;
      live++;
      if (J->phase == J_ITER) iter.push_back(J);
    }
    if (!live) return VFS_OK;
    if (iter.empty()) {
      // only checks and closes in flight: poll them, wait if none moved
      int moved = 0;
      for (Job* J : jobs) if (J->phase == J_CHECK || J->phase == J_POST) moved += job_advance_any(ctx, *J);
      if (!moved) wait_any(jobs);
      ticked_prev = false;
      continue;
    }
    bool need = !bg.exec || iter.size() * 2 < bg.members.size();
    for (Job* J : iter) {
      if (std::find(bg.members.begin(), bg.members.end(), J) == bg.members.end()) need = true;
    }
    if (need) {
      int r = batch_capture(ctx, s0, fork, joins, iter, bg);
      if (r) return r;
    }
    // order the tick after every member's out-of-graph work
    for (Job* J : bg.members) {
      if (!J->pending) continue;
      CK(cudaEventRecord(J->g->ev_pend, J->g->s));
      CK(cudaStreamWaitEvent(s0, J->g->ev_pend, 0));
      J->pending = false;
    }
    CK(cudaGraphLaunch(bg.exec, s0));
    g_launches += bg.kernels;
    cudaEvent_t tick = ticks[t & 1];
    CK(cudaEventRecord(tick, s0));
    const bool have_prev = ticked_prev;
    if (have_prev) CK(cudaEventSynchronize(ticks[(t - 1) & 1]));
    for (Job* J : bg.members) {
      if (J->phase != J_ITER) continue;
      const int r = J->mixed() ? batch_after_tick<float>(ctx, *J, tick, have_prev)
                               : batch_after_tick<double>(ctx, *J, tick, have_prev);
      if (r) job_fail(ctx, *J, r);
    }
    // checks and closes of other grids progress between ticks
    for (Job* J : jobs) {
      if (J->phase != J_CHECK && J->phase != J_POST) continue;
      CK(cudaStreamWaitEvent(J->g->s, tick, 0));
      job_advance_any(ctx, *J);
    }
    ticked_prev = true;
    t++;
  }
}

int do_solve(vfs_ctx* ctx, Grid& g, const vfs_solve_params* p, vfs_solve_info* info) {
  int r = check_params(ctx, p);
  if (r) return r;
  if (!g.lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs must run before the solve");
  if (g.m && p->restart > g.m) return fail(ctx, VFS_ERR_ARG, "restart length cannot grow after the first solve");
  Job J;
  J.g = &g;
  J.p = *p;
  std::vector<Job*> jobs{&J};
  r = run_jobs_streams(ctx, jobs);
  if (r) return r;
  if (J.rc) return J.rc;
  if (info) *info = J.info;
  return VFS_OK;
}

// Host-side nvert of the finest level: fluid count, the byte copy the
// integer nvert tests use (when every value is an integer in [0, 127]), and
// the upload.  The grid's other derived fields follow in grid_derive.
int grid_set_nvert(vfs_ctx* ctx, Grid& g, const double* nvert) {
  const Dims& d = g.d;
  const size_t N = ncell(d);
  g.nfluid = 0.;
  for (int k = 1; k < d.mz - 1; k++)
    for (int j = 1; j < d.my - 1; j++)
      for (int i = 1; i < d.mx - 1; i++)
        if (nvert[cidx(d, i, j, k)] < 0.1) g.nfluid += 1.;
  std::vector<uint8_t> nbh(N);
  bool integral = true;
  for (size_t c = 0; c < N && integral; c++) {
    const double v = nvert[c];
    integral = v >= 0. && v <= 127. && v == (double)(int)v;
    nbh[c] = integral ? (uint8_t)(int)v : 0;
  }
  Level& F = g.lev[g.L - 1];
  CK(cudaMemcpyAsync(F.nvert, nvert, N * sizeof(double), cudaMemcpyHostToDevice, g.s));
  g.nb8 = nullptr;
  if (integral) {
    if (!g.nb8_buf) {
      const int r = galloc(ctx, g, &g.nb8_buf, N);
      if (r) return r;
    }
    CK(cudaMemcpyAsync(g.nb8_buf, nbh.data(), N, cudaMemcpyHostToDevice, g.s));
    g.nb8 = g.nb8_buf;
  }
  // the host vector must outlive the copies
  CK(cudaStreamSynchronize(g.s));
  return VFS_OK;
}

// Everything derived from the finest coordinates and nvert: coarse nodes and
// masks (every other node; MyNvertRestriction), the metrics of every level,
// the restriction weights and the inverse metric.  The operator is rebuilt
// by vfs_poisson_lhs.
int grid_derive(vfs_ctx* ctx, Grid& g) {
  const int L = g.L;
  for (int l = L - 2; l >= 0; l--)
    launch_coarsen(g.lev[l + 1].d, g.lev[l].d, g.si, g.sj, g.sk, g.lev[l + 1].coor, g.lev[l + 1].nvert, g.lev[l].coor,
                   g.lev[l].nvert, g.s);
  for (int l = 0; l < L; l++) launch_form_metrics(g.lev[l].d, g.lev[l].coor, g.lev[l].M, g.mtmp, g.s);
  for (int l = 0; l < L; l++) launch_restrict_weights(g.lev[l].N, g.lev[l].nvert, g.lev[l].rw32, g.lev[l].rw64, g.s);
  Level& F = g.lev[L - 1];
  launch_inverse_metric(F.d, F.M, F.nvert, g.minv, g.s);
  cudaError_t e = cudaStreamSynchronize(g.s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "grid setup");
  // the operator and every captured iteration depend on these
  g.lhs = false;
  if (g.ig_exec) {
    cudaGraphExecDestroy(g.ig_exec);
    g.ig_exec = nullptr;
  }
  return VFS_OK;
}

size_t level_bytes(const Dims& d, bool finest) {
  const size_t N = ncell(d);
  size_t b = N * (3 + 1 + MP_TOTAL + 19 + 19 + 1 + 1) * 8 + N * (19 + 1 + 1) * 4 + N;  // coor nvert M coef mcoef lf64 rw64 mcoef32 lf32 rw32 pcode
  b += 19 * 2 * hslot(d) + N * (4 + 4 + 4);  // hcoef lfh rwh, and dinvh (finest) or dvalh (coarsest)
  b += N * (8 + 8 + 4 + 4 + 16);              // face form: ffi ffk ffj faj (with the code bits), ffc
  b += N * (3 * 4 + 3 * 8);                                            // MG work vectors, both precisions
  if (finest) b += N * 8 * (9 + 9 + 9 + 3 + 3 + 3 + 3 + 3) + N * 3;  // pd pw minv u ustar p phi b ucat aos, nb8 pc
  return b;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

void vfs_default_params(vfs_solve_params* p) {
  if (!p) return;
  p->precision = VFS_MIXED;
  p->rtol = 1e-9;
  p->maxit = 200;
  p->restart = 30;
  p->nu1 = 3;
  p->nu2 = 3;
  p->omega = 0.9;
  p->smoother = VFS_SMOOTH_CHEBYSHEV;
  p->cheb_hi = 2.0;
  p->cheb_ratio = 6.0;
  p->warm_start = 0;
  p->div_tol = 0.;
  p->orth = VFS_ORTH_CGS;
  p->smooth_cols = 0;
  p->nu1_coarse = -1;
  p->nu2_coarse = -1;
  p->mg_half = 0;
  p->proj_exact = 0;
  p->mg_grouped = 0;
  p->mg_stage = STAGE_REGS;
}

int vfs_create(const vfs_config* cfg, vfs_ctx** out) {
  if (!out) return VFS_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return VFS_ERR_CUDA;
  }
  vfs_ctx* ctx = new vfs_ctx();
  ctx->device = cfg ? cfg->device : 0;
  ctx->budget = cfg ? (size_t)cfg->hbm_budget_bytes : 0;
  ctx->max_inflight = (cfg && cfg->max_inflight > 0) ? cfg->max_inflight : 16;
  if (ctx->device < 0 || ctx->device >= ndev) {
    delete ctx;
    return VFS_ERR_ARG;
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess) {
    delete ctx;
    return VFS_ERR_CUDA;
  }
  *out = ctx;
  return VFS_OK;
}

void vfs_destroy(vfs_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  for (auto& e : ctx->marks) cudaEventDestroy(e);
  ctx->inflight.clear();  // grid_free below waits for each grid's stream
  for (auto& kv : ctx->grids) grid_free(ctx, kv.second);
  ctx->grids.clear();
  if (ctx->s0) cudaStreamDestroy(ctx->s0);
  delete ctx;
}

const char* vfs_last_error(const vfs_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int vfs_grid_estimate(const vfs_grid_desc* desc, int restart, unsigned long long* bytes) {
  if (!desc || !bytes) return VFS_ERR_ARG;
  Dims d{desc->mx, desc->my, desc->mz, desc->i_periodic, desc->j_periodic, desc->k_periodic};
  size_t b = level_bytes(d, true);
  Dims c = d;
  for (int l = 1; l < desc->mg_levels; l++) {
    if (!desc->semi_i) c.mx = (c.mx - 2) / 2 + 2;
    if (!desc->semi_j) c.my = (c.my - 2) / 2 + 2;
    if (!desc->semi_k) c.mz = (c.mz - 2) / 2 + 2;
    b += level_bytes(c, false);
  }
  const size_t N = ncell(d);
  b += N * 8 * (size_t)(restart + 2) + N * 4 * (size_t)restart + N * 8 * (size_t)restart;
  *bytes = b;
  return VFS_OK;
}

int vfs_grid_create(vfs_ctx* ctx, const vfs_grid_desc* desc, int* grid_id) {
  if (!ctx) return VFS_ERR_ARG;
  if (!desc || !grid_id || !desc->coor || !desc->nvert) return fail(ctx, VFS_ERR_ARG, "null grid description");
  CK(cudaSetDevice(ctx->device));
  const int L = desc->mg_levels;
  if (L < 1 || L > MAXLEV) return fail(ctx, VFS_ERR_ARG, "mg_levels must be in [1, 12]");
  Dims d{desc->mx, desc->my, desc->mz, desc->i_periodic ? 1 : 0, desc->j_periodic ? 1 : 0, desc->k_periodic ? 1 : 0};
  const int sem[3] = {desc->semi_i, desc->semi_j, desc->semi_k};
  const int ext[3] = {d.mx - 2, d.my - 2, d.mz - 2};
  const int per[3] = {d.ip, d.jp, d.kp};
  for (int a = 0; a < 3; a++) {
    int n = ext[a];
    if (n < 2) return fail(ctx, VFS_ERR_ARG, "every axis needs at least 2 interior cells");
    for (int l = 1; l < L; l++) {
      if (sem[a]) continue;
      if (n % 2) return fail(ctx, VFS_ERR_ARG, "a coarsened axis has an odd cell count at some level");
      n = coarse_n(n);
    }
    if (per[a] && n < 3) return fail(ctx, VFS_ERR_ARG, "a periodic axis needs at least 3 cells on the coarsest level");
    if (n < 2) return fail(ctx, VFS_ERR_ARG, "too many multigrid levels for this grid");
  }
  if (ext[1] > 3000) return fail(ctx, VFS_ERR_ARG, "the y-line smoother supports at most 3000 cells in j");
  if ((double)(ext[0] + 2) * (ext[1] + 2) * (ext[2] + 2) > 2147483647.)
    return fail(ctx, VFS_ERR_ARG, "a grid holds at most 2^31 - 1 cells including ghosts");
  Grid* gp = new Grid();
  Grid& g = *gp;
  g.d = d;
  g.L = L;
  g.si = desc->semi_i ? 1 : 0;
  g.sj = desc->semi_j ? 1 : 0;
  g.sk = desc->semi_k ? 1 : 0;
  g.immersed = desc->immersed;
  auto bail = [&](int r) {
    grid_free(ctx, gp);
    return r;
  };
  if (cudaStreamCreateWithFlags(&g.s, cudaStreamNonBlocking) != cudaSuccess) return bail(cuda_fail(ctx, cudaGetLastError(), "stream"));
  cudaEventCreateWithFlags(&g.ev[0], cudaEventDisableTiming);
  cudaEventCreateWithFlags(&g.ev[1], cudaEventDisableTiming);
  cudaEventCreate(&g.t0);
  cudaEventCreate(&g.t1);
  if (cudaMallocHost(&g.hstat, 4 * sizeof(int)) != cudaSuccess || cudaMallocHost(&g.hk, sizeof(KrylovState)) != cudaSuccess ||
      cudaMallocHost(&g.hv, 4 * sizeof(double)) != cudaSuccess)
    return bail(cuda_fail(ctx, cudaGetLastError(), "pinned"));
  cudaEventCreateWithFlags(&g.ev_chk, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&g.ev_done, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&g.ev_pend, cudaEventDisableTiming);
  for (cudaEvent_t* e : {&g.ev_pin, &g.ev_p, &g.ev_u, &g.ev_cs, &g.ev_uin})
    cudaEventCreateWithFlags(e, cudaEventDisableTiming);
  if (cudaStreamCreateWithFlags(&g.cs, cudaStreamNonBlocking) != cudaSuccess)
    return bail(cuda_fail(ctx, cudaGetLastError(), "stream"));
  // level extents, finest = L-1
  g.lev[L - 1].d = d;
  for (int l = L - 2; l >= 0; l--) {
    Dims c = g.lev[l + 1].d;
    if (!g.si) c.mx = coarse_n(c.mx - 2) + 2;
    if (!g.sj) c.my = coarse_n(c.my - 2) + 2;
    if (!g.sk) c.mz = coarse_n(c.mz - 2) + 2;
    g.lev[l].d = c;
  }
  int r;
  double* tmp = nullptr;
  for (int l = 0; l < L; l++) {
    Level& Lv = g.lev[l];
    Lv.N = ncell(Lv.d);
#define GAB(ptr, cnt)                                           \
  do {                                                          \
    r = galloc(ctx, g, &(ptr), (size_t)(cnt));                  \
    if (r) return bail(r);                                      \
  } while (0)
    GAB(Lv.coor, 3 * Lv.N);
    GAB(Lv.nvert, Lv.N);
    GAB(Lv.M, MP_TOTAL * Lv.N);
    GAB(Lv.coef, 19 * Lv.N);
    GAB(Lv.mcoef, 19 * Lv.N);
    GAB(Lv.mcoef32, 19 * Lv.N);
    GAB(Lv.lf32, Lv.N);
    GAB(Lv.lf64, Lv.N);
    GAB(Lv.rw32, Lv.N);
    GAB(Lv.rw64, Lv.N);
    if (l > 0) GAB(Lv.pcode, Lv.N);
    GAB(Lv.hcoef, 19 * hslot(Lv.d));
    GAB(Lv.ffi, Lv.N);
    GAB(Lv.ffk, Lv.N);
    GAB(Lv.ffj, Lv.N);
    GAB(Lv.faj, Lv.N);
    GAB(Lv.ffc, Lv.N);
    GAB(Lv.lfh, Lv.N);
    GAB(Lv.rwh, Lv.N);
    if (l == L - 1) GAB(Lv.dinvh, Lv.N);
    if (l == 0) GAB(Lv.dvalh, Lv.N);
  }
  const size_t N = ncell(d);
  GAB(tmp, 9 * N);
  GAB(g.pd, 9 * N);
  GAB(g.pw, 9 * N);
  GAB(g.pc, N);
  GAB(g.minv, 9 * N);
  GAB(g.u, 3 * N);
  GAB(g.ustar, 3 * N);
  GAB(g.p, N);
  GAB(g.phi, N);
  GAB(g.b, N);
  GAB(g.bs, N);
  GAB(g.ucat, 3 * N);
  GAB(g.aos, 3 * N);
  GAB(g.parts, (size_t)krylov_nblocks(N) * 72 + 4096);
  GAB(g.scal, 64);
  g.mtmp = tmp;
  Level& F = g.lev[L - 1];
  if (cudaMemcpyAsync(F.coor, desc->coor, 3 * N * sizeof(double), cudaMemcpyHostToDevice, g.s) != cudaSuccess)
    return bail(cuda_fail(ctx, cudaGetLastError(), "upload"));
  r = grid_set_nvert(ctx, g, desc->nvert);
  if (!r) r = grid_derive(ctx, g);
  if (r) return bail(r);
  const int id = ctx->next_id++;
  ctx->grids[id] = gp;
  *grid_id = id;
  return VFS_OK;
}

int vfs_grid_destroy(vfs_ctx* ctx, int grid) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* g = get_grid(ctx, grid);
  if (!g) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (g->busy) return fail(ctx, VFS_ERR_BUSY, "the grid has a request in flight");
  grid_free(ctx, g);
  ctx->grids.erase(grid);
  return VFS_OK;
}

int vfs_grid_update_nvert(vfs_ctx* ctx, int grid, const double* nvert) {
  if (!ctx || !nvert) return VFS_ERR_ARG;
  Grid* g = get_grid(ctx, grid);
  if (!g) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (g->busy) return fail(ctx, VFS_ERR_BUSY, "the grid has a request in flight");
  CK(cudaSetDevice(ctx->device));
  int r = grid_set_nvert(ctx, *g, nvert);
  if (!r) r = grid_derive(ctx, *g);
  return r;
}

int vfs_grid_update_coords(vfs_ctx* ctx, int grid, const double* coor) {
  if (!ctx || !coor) return VFS_ERR_ARG;
  Grid* g = get_grid(ctx, grid);
  if (!g) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (g->busy) return fail(ctx, VFS_ERR_BUSY, "the grid has a request in flight");
  CK(cudaSetDevice(ctx->device));
  Level& F = g->lev[g->L - 1];
  CK(cudaMemcpyAsync(F.coor, coor, 3 * ncell(g->d) * sizeof(double), cudaMemcpyHostToDevice, g->s));
  return grid_derive(ctx, *g);
}

namespace {
constexpr int PETSC_VEC_CLASSID = 1211214;
void put_be32(unsigned char* p, uint32_t v) {
  for (int b = 0; b < 4; b++) p[b] = (unsigned char)(v >> (24 - 8 * b));
}
uint32_t get_be32(const unsigned char* p) {
  uint32_t v = 0;
  for (int b = 0; b < 4; b++) v = (v << 8) | p[b];
  return v;
}
}  // namespace

int vfs_petsc_vec_read(const char* path, double* out, long long n, long long* n_file) {
  if (!path) return VFS_ERR_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return VFS_ERR_IO;
  unsigned char hdr[8];
  if (std::fread(hdr, 1, 8, f) != 8 || (int)get_be32(hdr) != PETSC_VEC_CLASSID) {
    std::fclose(f);
    return VFS_ERR_IO;
  }
  const long long len = (long long)(int32_t)get_be32(hdr + 4);
  if (n_file) *n_file = len;
  if (!out) {
    std::fclose(f);
    return len >= 0 ? VFS_OK : VFS_ERR_IO;
  }
  if (len != n) {
    std::fclose(f);
    return VFS_ERR_ARG;
  }
  std::vector<unsigned char> buf(1 << 20);
  long long done = 0;
  while (done < n) {
    const size_t want = (size_t)std::min<long long>(n - done, (long long)(buf.size() / 8));
    if (std::fread(buf.data(), 8, want, f) != want) {
      std::fclose(f);
      return VFS_ERR_IO;
    }
    for (size_t q = 0; q < want; q++) {
      uint64_t v = 0;
      for (int b = 0; b < 8; b++) v = (v << 8) | buf[8 * q + b];
      std::memcpy(out + done + q, &v, 8);
    }
    done += (long long)want;
  }
  std::fclose(f);
  return VFS_OK;
}

int vfs_petsc_vec_write(const char* path, const double* in, long long n) {
  if (!path || (n > 0 && !in) || n < 0 || n > 2147483647LL) return VFS_ERR_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return VFS_ERR_IO;
  unsigned char hdr[8];
  put_be32(hdr, (uint32_t)PETSC_VEC_CLASSID);
  put_be32(hdr + 4, (uint32_t)n);
  bool ok = std::fwrite(hdr, 1, 8, f) == 8;
  std::vector<unsigned char> buf(1 << 20);
  long long done = 0;
  while (ok && done < n) {
    const size_t m = (size_t)std::min<long long>(n - done, (long long)(buf.size() / 8));
    for (size_t q = 0; q < m; q++) {
      uint64_t v;
      std::memcpy(&v, in + done + q, 8);
      for (int b = 0; b < 8; b++) buf[8 * q + b] = (unsigned char)(v >> (56 - 8 * b));
    }
    ok = std::fwrite(buf.data(), 8, m, f) == m;
    done += (long long)m;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? VFS_OK : VFS_ERR_IO;
}

int vfs_grid_bytes(vfs_ctx* ctx, int grid, unsigned long long* bytes) {
  if (!ctx || !bytes) return VFS_ERR_ARG;
  Grid* g = get_grid(ctx, grid);
  if (!g) return fail(ctx, VFS_ERR_ARG, "no such grid");
  *bytes = g->bytes;
  return VFS_OK;
}

int vfs_poisson_lhs(vfs_ctx* ctx, int grid) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  CK(cudaSetDevice(ctx->device));
  const size_t N = ncell(g.d);
  double* gt = nullptr;
  unsigned* dmask = nullptr;
  CK(cudaMalloc(&gt, 9 * N * sizeof(double)));
  CK(cudaMalloc(&dmask, 2 * sizeof(unsigned)));
  CK(cudaMemsetAsync(dmask + 1, 0, sizeof(unsigned), g.s));
  for (int l = 0; l < g.L; l++) {
    Level& Lv = g.lev[l];
    launch_gtensor(Lv.d, Lv.M, gt, g.s);
    launch_assemble(Lv.d, gt, Lv.nvert, Lv.M + Lv.N * MP_AJ, Lv.coef, Lv.mcoef, Lv.mcoef32, dmask, g.s);
    launch_face_operator(Lv.d, gt, Lv.nvert, Lv.M + Lv.N * MP_AJ, Lv.ffi, Lv.ffk, Lv.ffj, Lv.faj, Lv.ffc, g.s);
    CK(cudaMemcpyAsync(&Lv.mask, dmask, sizeof(unsigned), cudaMemcpyDeviceToHost, g.s));
    if (l > 0) launch_prolong_codes(Lv.d, g.lev[l - 1].d, g.si, g.sj, g.sk, Lv.nvert, g.lev[l - 1].nvert, Lv.pcode, g.s);
    launch_line_factors<float>(Lv.d, Lv.mcoef, Lv.lf32, g.s);
    launch_line_factors<double>(Lv.d, Lv.mcoef, Lv.lf64, g.s);
    launch_half_operator(Lv.d, Lv.mcoef, Lv.hcoef, l == g.L - 1 ? Lv.dinvh : nullptr, l == 0 ? Lv.dvalh : nullptr,
                         dmask + 1, g.s);
    launch_line_factors_half(Lv.d, Lv.hcoef, Lv.mcoef, Lv.lfh, g.s);
  }
  CK(cudaMemsetAsync(g.lev[0].rwh, 0, g.lev[0].N * sizeof(float), g.s));
  for (int l = 1; l < g.L; l++)
    launch_restrict_weights_half(g.lev[l].d, g.lev[l - 1].d, g.si, g.sj, g.sk, g.lev[l].nvert, g.lev[l].mcoef,
                                 g.lev[l - 1].mcoef, g.lev[l].rwh, g.s);
  Level& F = g.lev[g.L - 1];
  launch_proj_dots(F.d, F.M, g.pd, g.s);
  launch_proj_weights(F.d, g.pd, F.M, F.nvert, g.pw, g.pc, g.s);
  unsigned range = 0;
  CK(cudaMemcpyAsync(&range, dmask + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, g.s));
  CK(cudaStreamSynchronize(g.s));
  g.half_ok = range == 0;
  cudaFree(gt);
  cudaFree(dmask);
  // connected fluid regions of the finest level: one null vector each
  {
    std::vector<double> nv(N);
    CK(cudaMemcpy(nv.data(), F.nvert, N * sizeof(double), cudaMemcpyDeviceToHost));
    std::vector<char> fl(N, 0);
    bool solid = false;
    for (int k = 1; k < F.d.mz - 1; k++)
      for (int j = 1; j < F.d.my - 1; j++)
        for (int i = 1; i < F.d.mx - 1; i++) {
          const size_t c = cidx(F.d, i, j, k);
          fl[c] = nv[c] < 0.1;
          solid = solid || !fl[c];
        }
    std::vector<int> lab;
    g.ncomp = solid ? fluid_regions(F.d, fl, lab) : 1;
    if (g.ncomp > 1) {
      if (!g.comp) {
        const int r = galloc(ctx, g, &g.comp, N);
        if (r) return r;
      }
      CK(cudaMemcpy(g.comp, lab.data(), N * sizeof(int), cudaMemcpyHostToDevice));
    }
  }
  // coarsest level: dense inverse of A + sigma e e^T when small enough
  Level& C = g.lev[0];
  const int n = (C.d.mx - 2) * (C.d.my - 2) * (C.d.mz - 2);
  if (g.ig_exec) {  // the slot set or the coarse solve may change
    cudaGraphExecDestroy(g.ig_exec);
    g.ig_exec = nullptr;
  }
  C.nco = 0;
  if (n <= DENSE_MAX) {
    std::vector<double> cp(C.N);
    CK(cudaMemcpy(cp.data(), C.mcoef, C.N * sizeof(double), cudaMemcpyDeviceToHost));
    double sabs = 0.;
    long nf = 0;
    for (size_t c = 0; c < C.N; c++)
      if (cp[c] != 0.) {
        sabs += std::fabs(cp[c]);
        nf++;
      }
    g.ncomp_c = 1;
    int* ccomp = nullptr;
    if (nf > 0) {
      // the level's fluid rows (nonzero centre coefficient) and their regions
      std::vector<char> fl(C.N, 0);
      for (int k = 1; k < C.d.mz - 1; k++)
        for (int j = 1; j < C.d.my - 1; j++)
          for (int i = 1; i < C.d.mx - 1; i++) fl[cidx(C.d, i, j, k)] = cp[cidx(C.d, i, j, k)] != 0.;
      std::vector<int> lab;
      g.ncomp_c = fluid_regions(C.d, fl, lab);
      if (g.ncomp_c > 1) {
        CK(cudaMalloc(&ccomp, C.N * sizeof(int)));
        CK(cudaMemcpy(ccomp, lab.data(), C.N * sizeof(int), cudaMemcpyHostToDevice));
      }
    }
    if (nf > 0) {
      const double sigma = -(sabs / nf) / (double)nf;
      double *W = nullptr, *fac = nullptr, *pval = nullptr;
      int* piv = nullptr;
      CK(cudaMalloc(&W, (size_t)n * 2 * n * sizeof(double)));
      CK(cudaMalloc(&fac, (size_t)n * sizeof(double)));
      CK(cudaMalloc(&pval, sizeof(double)));
      CK(cudaMalloc(&piv, sizeof(int)));
      int r = C.Binv ? VFS_OK : galloc(ctx, g, &C.Binv, (size_t)n * n);
      if (!r && !C.Binv32) r = galloc(ctx, g, &C.Binv32, (size_t)n * n);
      if (r) {
        cudaFree(W); cudaFree(fac); cudaFree(pval); cudaFree(piv); cudaFree(ccomp);
        return r;
      }
      launch_dense_inverse(C.d, C.mcoef, sigma, W, fac, piv, pval, C.Binv, C.Binv32, n, g.s, ccomp);
      cudaError_t e = cudaStreamSynchronize(g.s);
      cudaFree(W); cudaFree(fac); cudaFree(pval); cudaFree(piv); cudaFree(ccomp);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "coarse inverse");
      C.nco = n;
    }
  }
  g.lhs = true;
  return VFS_OK;
}

int vfs_set_field(vfs_ctx* ctx, int grid, int field, const double* host) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp || !host) return fail(ctx, VFS_ERR_ARG, "no such grid or null buffer");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  const size_t N = ncell(g.d);
  switch (field) {
    case VFS_FIELD_UCONT:
    case VFS_FIELD_USTAR: {
      double* dst = field == VFS_FIELD_UCONT ? g.u : g.ustar;
      CK(cudaMemcpyAsync(g.aos, host, 3 * N * sizeof(double), cudaMemcpyHostToDevice, g.s));
      launch_aos2soa(N, g.aos, dst, dst + N, dst + 2 * N, g.s);
      break;
    }
    case VFS_FIELD_P: CK(cudaMemcpyAsync(g.p, host, N * sizeof(double), cudaMemcpyHostToDevice, g.s)); break;
    case VFS_FIELD_PHI: CK(cudaMemcpyAsync(g.phi, host, N * sizeof(double), cudaMemcpyHostToDevice, g.s)); break;
    case VFS_FIELD_RHS: CK(cudaMemcpyAsync(g.b, host, N * sizeof(double), cudaMemcpyHostToDevice, g.s)); break;
    default: return fail(ctx, VFS_ERR_ARG, "field cannot be set");
  }
  CK(cudaStreamSynchronize(g.s));
  return VFS_OK;
}

int vfs_get_field(vfs_ctx* ctx, int grid, int field, double* host) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp || !host) return fail(ctx, VFS_ERR_ARG, "no such grid or null buffer");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  const size_t N = ncell(g.d);
  switch (field) {
    case VFS_FIELD_UCONT:
    case VFS_FIELD_USTAR: {
      double* src = field == VFS_FIELD_UCONT ? g.u : g.ustar;
      launch_soa2aos(N, src, src + N, src + 2 * N, g.aos, g.s);
      CK(cudaMemcpyAsync(host, g.aos, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, g.s));
      break;
    }
    case VFS_FIELD_P: CK(cudaMemcpyAsync(host, g.p, N * sizeof(double), cudaMemcpyDeviceToHost, g.s)); break;
    case VFS_FIELD_PHI: CK(cudaMemcpyAsync(host, g.phi, N * sizeof(double), cudaMemcpyDeviceToHost, g.s)); break;
    case VFS_FIELD_RHS: CK(cudaMemcpyAsync(host, g.b, N * sizeof(double), cudaMemcpyDeviceToHost, g.s)); break;
    case VFS_FIELD_UCAT: CK(cudaMemcpyAsync(host, g.ucat, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, g.s)); break;
    case VFS_FIELD_NVERT:
      CK(cudaMemcpyAsync(host, g.lev[g.L - 1].nvert, N * sizeof(double), cudaMemcpyDeviceToHost, g.s));
      break;
    default: return fail(ctx, VFS_ERR_ARG, "unknown field");
  }
  CK(cudaStreamSynchronize(g.s));
  return VFS_OK;
}

int vfs_volume_flux(vfs_ctx* ctx, int grid, double out[4]) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  Level& F = g.lev[g.L - 1];
  launch_volume_flux(F.d, g.immersed ? 1 : 0, g.U(), F.nvert, F.M, g.parts, g.scal, g.s, g.nb8);
  if (out) CK(cudaMemcpyAsync(out, g.scal, 4 * sizeof(double), cudaMemcpyDeviceToHost, g.s));
  CK(cudaStreamSynchronize(g.s));
  return VFS_OK;
}

int vfs_poisson_rhs(vfs_ctx* ctx, int grid, double dt, double st, double coeff, int meanfix, double* sum_out) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (int r_ = check_idle(ctx, gp)) return r_;
  if (!(dt > 0.)) return fail(ctx, VFS_ERR_ARG, "dt must be > 0");
  Grid& g = *gp;
  Level& F = g.lev[g.L - 1];
  g.dt = dt;
  g.st_ = st;
  g.coeff = coeff;
  launch_rhs(F.d, g.U(), F.nvert, dt, st, coeff, meanfix, g.b, g.parts, g.scal + 4, g.s, g.comp, g.ncomp);
  double sc[2];
  CK(cudaMemcpyAsync(sc, g.scal + 4, 2 * sizeof(double), cudaMemcpyDeviceToHost, g.s));
  CK(cudaStreamSynchronize(g.s));
  if (sum_out) *sum_out = sc[0];
  if (!(sc[0] == sc[0])) return fail(ctx, VFS_ERR_NUMERIC, "NaN in the right-hand side");
  return VFS_OK;
}

int vfs_poisson_solve(vfs_ctx* ctx, int grid, const vfs_solve_params* p, vfs_solve_info* info) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (int r_ = check_idle(ctx, gp)) return r_;
  vfs_solve_info tmp{};
  int r = do_solve(ctx, *gp, p, info ? info : &tmp);
  if (r) return r;
  const vfs_solve_info& i = info ? *info : tmp;
  if (!i.converged) return fail(ctx, VFS_ERR_NOTCONV, "FGMRES stopped at maxit above rtol");
  return VFS_OK;
}

int vfs_update_pressure(vfs_ctx* ctx, int grid) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  Level& F = g.lev[g.L - 1];
  launch_update_pressure(F.d, F.nvert, g.phi, g.p, g.s);
  CK(cudaStreamSynchronize(g.s));
  return VFS_OK;
}

int vfs_projection(vfs_ctx* ctx, int grid, double dt, double st, double coeff) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  if (!g.lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs must run before the projection");
  Level& F = g.lev[g.L - 1];
  launch_projection(F.d, g.pd, F.M, F.nvert, g.nb8, g.phi, dt, st, coeff, g.U(), g.s);
  launch_contra2cart(F.d, g.minv, F.nvert, g.U(), g.ucat, g.s);
  CK(cudaStreamSynchronize(g.s));
  return VFS_OK;
}

int vfs_projection_faces(vfs_ctx* ctx, int grid, double dt, double st, double coeff) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  if (!g.lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs must run before the projection");
  Level& F = g.lev[g.L - 1];
  launch_projection_fast(F.d, g.pw, g.pc, g.phi, dt, st, coeff, g.U(), g.s);
  launch_contra2cart(F.d, g.minv, F.nvert, g.U(), g.ucat, g.s);
  CK(cudaStreamSynchronize(g.s));
  return VFS_OK;
}

int vfs_divergence_max_noalloc(int device, int mx, int my, int mz, int i_periodic, int j_periodic, int k_periodic,
                               const double* ucont_x, const double* ucont_y, const double* ucont_z, const double* aj,
                               const double* nvert, double* out, void* stream, char* err, int err_len) {
  auto report = [&](int rc, const char* msg) {
    if (err && err_len > 0) {
      std::strncpy(err, msg, (size_t)err_len - 1);
      err[err_len - 1] = 0;
    }
    return rc;
  };
  if (!ucont_x || !ucont_y || !ucont_z || !aj || !nvert || !out) return report(VFS_ERR_ARG, "null device pointer");
  if (mx < 3 || my < 3 || mz < 3) return report(VFS_ERR_ARG, "every extent must be at least 3 (one interior cell)");
  if ((double)mx * my * mz > 2147483647.)
    return report(VFS_ERR_ARG, "a grid holds at most 2^31 - 1 cells including ghosts");
  Dims d{mx, my, mz, i_periodic ? 1 : 0, j_periodic ? 1 : 0, k_periodic ? 1 : 0};
  Ucont u{const_cast<double*>(ucont_x), const_cast<double*>(ucont_y), const_cast<double*>(ucont_z)};
  const char* why = "";
  const int rc = divergence_max_static(device, d, u, aj, nvert, out, (cudaStream_t)stream, &why);
  if (rc) return report(rc == 1 ? VFS_ERR_ARG : VFS_ERR_CUDA, why);
  return report(VFS_OK, "");
}

int vfs_divergence_max(vfs_ctx* ctx, int grid, double* out) {
  if (!ctx || !out) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  Level& F = g.lev[g.L - 1];
  launch_divergence(F.d, g.U(), F.M + F.N * MP_AJ, F.nvert, g.parts, g.scal + 8, g.s, g.nb8);
  CK(cudaMemcpyAsync(out, g.scal + 8, sizeof(double), cudaMemcpyDeviceToHost, g.s));
  CK(cudaStreamSynchronize(g.s));
  return VFS_OK;
}

}  // extern "C"

namespace {

// Everything of one projection step after the inputs are resident, up to the
// solve start (flux balance, RHS).
void step_pre(Grid& g, double dt, double st, double coeff) {
  Level& F = g.lev[g.L - 1];
  g.dt = dt;
  g.st_ = st;
  g.coeff = coeff;
  const double N = (double)ncell(F.d), nvb = g.nb8 ? 1.0 : 8.0;
  {
    // two passes over the fluid mask (the interface faces' fluxes and metric
    // norms are few)
    Probed pr(VFS_PROBE_ALL, g.s, "k_vflux (2 passes)", g.L - 1, 2.0 * N * nvb);
    dbg("volume_flux", 0, launch_volume_flux(F.d, g.immersed ? 1 : 0, g.U(), F.nvert, F.M, g.parts, g.scal, g.s, g.nb8),
        g.s);
  }
  {
    // U (3 components) and nvert read, b written; the mean fix reads nvert and
    // b and writes b
    Probed pr(VFS_PROBE_ALL, g.s, "k_rhs + k_meanfix", g.L - 1, N * (40.0 + 24.0 * g.ncomp));
    dbg("rhs", 0, launch_rhs(F.d, g.U(), F.nvert, dt, st, coeff, 1, g.b, g.parts, g.scal + 4, g.s, g.comp, g.ncomp),
        g.s);
  }
}
// After the solve: pressure, projection, Contra2Cart, divergence.
// Host outputs (nullable) leave on the grid's copy stream as soon as their
// data is final: the pressure right after its update (overlapping the
// projection), the corrected fluxes right after the projection (overlapping
// Contra2Cart and the divergence check); the main stream then waits for the
// copies.  p_in_pending: the pressure upload of the step (on the copy
// stream, overlapping the solve) must land before the update.
int step_post(Grid& g, double dt, double st, double coeff, bool exact, double* u_out, double* p_out,
              bool p_in_pending) {
  Level& F = g.lev[g.L - 1];
  const size_t N = ncell(g.d);
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t r) {
    if (r != cudaSuccess && e == cudaSuccess) e = r;
  };
  if (p_in_pending) ok(cudaStreamWaitEvent(g.s, g.ev_pin, 0));
  const double Nd = (double)N;
  {
    // nvert and phi read, p read and written
    Probed pr(VFS_PROBE_ALL, g.s, "k_update_p", g.L - 1, Nd * 32.0);
    dbg("update_pressure", 0, launch_update_pressure(F.d, F.nvert, g.phi, g.p, g.s), g.s);
  }
  // projection: the 9 metric products, 3 face Jacobians, nvert bytes (or
  // doubles) and phi read, U read and written; on face weights: the 9
  // weights, the code and phi read, U read and written
  const double proj_b = exact ? 9 * 8.0 + 24.0 + (g.nb8 ? 1.0 : 8.0) + 8.0 + 48.0 : 9 * 8.0 + 2.0 + 8.0 + 48.0;
  const char* proj_name = exact ? "k_projection" : "k_projection_fast";
  auto project = [&](int k0, int k1) {
    return exact ? launch_projection(F.d, g.pd, F.M, F.nvert, g.nb8, g.phi, dt, st, coeff, g.U(), g.s, k0, k1)
                 : launch_projection_fast(F.d, g.pw, g.pc, g.phi, dt, st, coeff, g.U(), g.s, k0, k1);
  };
  if (p_out) {
    ok(cudaEventRecord(g.ev_p, g.s));
    ok(cudaStreamWaitEvent(g.cs, g.ev_p, 0));
    ok(cudaMemcpyAsync(p_out, g.p, N * sizeof(double), cudaMemcpyDeviceToHost, g.cs));
  }
  if (!u_out) {
    Probed pr(VFS_PROBE_ALL, g.s, proj_name, g.L - 1, Nd * proj_b);
    dbg("projection", 0, project(0, -1), g.s);
  } else {
    // Interior planes in slabs: a slab is projected and converted to AoS on
    // the step stream and goes down on the copy stream while the next one
    // is projected; the k ghost planes (filled from planes mz-2 and 1)
    // follow the last slab.
    const int mz = F.d.mz;
    const size_t P = (size_t)F.d.mx * F.d.my;
    auto to_aos = [&](int k0, int k1) {
      const size_t c0 = k0 * P;
      launch_soa2aos((k1 - k0) * P, g.u + c0, g.u + N + c0, g.u + 2 * N + c0, g.aos + 3 * c0, g.s);
    };
    auto download = [&](int k0, int k1) {
      const size_t c0 = k0 * P;
      ok(cudaMemcpyAsync(u_out + 3 * c0, g.aos + 3 * c0, 3 * (k1 - k0) * P * sizeof(double), cudaMemcpyDeviceToHost,
                         g.cs));
    };
    const int inner = mz - 2;
    const int S = std::min(inner, transfer_slabs(N));
    for (int q = 0; q < S; q++) {
      const int k0 = 1 + (int)((long long)inner * q / S), k1 = 1 + (int)((long long)inner * (q + 1) / S);
      {
        Probed pr(VFS_PROBE_ALL, g.s, proj_name, g.L - 1, (double)(k1 - k0) * P * proj_b);
        dbg("projection", 0, project(k0, k1), g.s);
      }
      to_aos(k0, k1);
      ok(cudaEventRecord(g.ev_u, g.s));
      ok(cudaStreamWaitEvent(g.cs, g.ev_u, 0));
      download(k0, k1);
    }
    dbg("ucont_ghosts", 0, launch_ucont_ghosts(F.d, g.U(), 0, 1, g.s), g.s);
    dbg("ucont_ghosts", 0, launch_ucont_ghosts(F.d, g.U(), mz - 1, mz, g.s), g.s);
    to_aos(0, 1);
    to_aos(mz - 1, mz);
    ok(cudaEventRecord(g.ev_u, g.s));
    ok(cudaStreamWaitEvent(g.cs, g.ev_u, 0));
    download(0, 1);
    download(mz - 1, mz);
  }
  {
    // the inverse metric (9), nvert and U read, Ucat written
    Probed pr(VFS_PROBE_ALL, g.s, "k_contra2cart", g.L - 1, Nd * (72.0 + 8.0 + 24.0 + 24.0));
    dbg("contra2cart", 0, launch_contra2cart(F.d, g.minv, F.nvert, g.U(), g.ucat, g.s), g.s);
  }
  {
    // U, aj and the nvert bytes (or doubles) read
    Probed pr(VFS_PROBE_ALL, g.s, "k_divergence", g.L - 1, Nd * (24.0 + 8.0 + (g.nb8 ? 1.0 : 8.0)));
    dbg("divergence", 0, launch_divergence(F.d, g.U(), F.M + F.N * MP_AJ, F.nvert, g.parts, g.scal + 8, g.s, g.nb8),
        g.s);
  }
  if (p_out || u_out) {
    ok(cudaEventRecord(g.ev_cs, g.cs));
    ok(cudaStreamWaitEvent(g.s, g.ev_cs, 0));
  }
  return (int)e;
}

}  // namespace

extern "C" {

int vfs_projection_step(vfs_ctx* ctx, int grid, double* ucont_inout, double* p_inout, double dt, double st,
                        double coeff, const vfs_solve_params* p, vfs_solve_info* info, double* divmax) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  Grid& g = *gp;
  int r = check_params(ctx, p);
  if (r) return r;
  if (!g.lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs must run before the projection step");
  if (!(dt > 0.)) return fail(ctx, VFS_ERR_ARG, "dt must be > 0");
  if (g.m && p->restart > g.m) return fail(ctx, VFS_ERR_ARG, "restart length cannot grow after the first solve");
  if (g.busy) return fail(ctx, VFS_ERR_BUSY, "the grid has a request in flight");
  g.solo = false;  // requests share the GPU
  Job J;
  J.g = &g;
  J.p = *p;
  J.pre = J.post = true;
  J.u_in = ucont_inout;
  J.u_out = ucont_inout;
  J.p_in = p_inout;
  J.p_out = p_inout;
  J.dt = dt;
  J.st = st;
  J.coeff = coeff;
  std::vector<Job*> jobs{&J};
  r = run_jobs_streams(ctx, jobs);
  if (r) return r;
  if (J.rc) return fail(ctx, J.rc, J.err);
  if (info) *info = J.info;
  if (divmax) *divmax = J.divmax;
  if (!J.info.converged) return fail(ctx, VFS_ERR_NOTCONV, "FGMRES stopped at maxit above rtol");
  return VFS_OK;
}

int vfs_projection_step_batch(vfs_ctx* ctx, int n, const int* grids, double dt, double st, double coeff,
                              const vfs_solve_params* p, int n_params, vfs_solve_info* infos, double* divmax) {
  if (!ctx || n < 0 || (n && !grids) || !p) return VFS_ERR_ARG;
  if (n_params != 1 && n_params != n) return fail(ctx, VFS_ERR_ARG, "n_params must be 1 or n");
  if (!(dt > 0.)) return fail(ctx, VFS_ERR_ARG, "dt must be > 0");
  std::vector<Job> js(n);
  std::vector<Job*> jobs(n);
  for (int q = 0; q < n; q++) {
    const vfs_solve_params* pq = p + (n_params == 1 ? 0 : q);
    int r = check_params(ctx, pq);
    if (r) return r;
    Grid* g = get_grid(ctx, grids[q]);
    if (!g) return fail(ctx, VFS_ERR_ARG, "no such grid in the batch");
    if (!g->lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs must run before the batch");
    if (g->m && pq->restart > g->m) return fail(ctx, VFS_ERR_ARG, "restart cannot grow");
    if (g->busy) return fail(ctx, VFS_ERR_BUSY, "a grid of the batch has a request in flight");
    for (int u = 0; u < q; u++)
      if (grids[u] == grids[q]) return fail(ctx, VFS_ERR_ARG, "a grid appears twice in the batch");
    Job& J = js[q];
    J.g = g;
    J.p = *pq;
    J.pre = J.post = true;
    J.dt = dt;
    J.st = st;
    J.coeff = coeff;
    jobs[q] = &J;
  }
  if (!ctx->s0) CK(cudaStreamCreateWithFlags(&ctx->s0, cudaStreamNonBlocking));
  int r = run_jobs_batch(ctx, jobs, ctx->s0);
  if (r) return r;
  int rc = VFS_OK;
  for (int q = 0; q < n; q++) {
    if (js[q].rc) return fail(ctx, js[q].rc, js[q].err);
    if (infos) infos[q] = js[q].info;
    if (divmax) divmax[q] = js[q].divmax;
    if (!js[q].info.converged) rc = VFS_ERR_NOTCONV;
  }
  if (rc) fail(ctx, rc, "a solve of the batch stopped at maxit above rtol");
  return rc;
}

int vfs_submit(vfs_ctx* ctx, const vfs_request* req, long long* ticket) {
  if (!ctx || !req || !ticket) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, req->grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  Grid& g = *gp;
  int r = check_params(ctx, &req->params);
  if (r) return r;
  if (!g.lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs must run before a request");
  if (!(req->dt > 0.)) return fail(ctx, VFS_ERR_ARG, "dt must be > 0");
  if (g.m && req->params.restart > g.m) return fail(ctx, VFS_ERR_ARG, "restart length cannot grow");
  if (g.busy) return fail(ctx, VFS_ERR_BUSY, "the grid has a request in flight");
  if ((int)ctx->inflight.size() >= ctx->max_inflight) return fail(ctx, VFS_ERR_BUSY, "all request slots are in use");
  // admission against the HBM budget: the grid's solver memory is reserved now
  r = req->params.precision == VFS_MIXED ? ensure_mg<float>(ctx, g) : ensure_mg<double>(ctx, g);
  if (!r) r = ensure_krylov(ctx, g, req->params.restart, req->params.precision);
  if (r) return r;
  auto box = std::make_unique<vfs_job_box>();
  Job& J = box->job;
  J.g = &g;
  J.p = req->params;
  J.pre = J.post = true;
  J.u_in = req->ucont_in;
  J.u_out = req->ucont_out;
  J.p_in = req->p_in;
  J.p_out = req->p_out;
  J.dt = req->dt;
  J.st = req->st;
  J.coeff = req->coeff;
  J.ticket = ctx->next_ticket++;
  g.busy = J.ticket;
  job_advance_any(ctx, J);  // inputs and right-hand side go to the device now
  *ticket = J.ticket;
  ctx->inflight[J.ticket] = std::move(box);
  return VFS_OK;
}

int vfs_poll(vfs_ctx* ctx, int wait, vfs_result* out) {
  if (!ctx || !out) return VFS_ERR_ARG;
  for (;;) {
    for (auto it = ctx->inflight.begin(); it != ctx->inflight.end(); ++it) {
      Job& J = it->second->job;
      if (J.phase != J_DONE) continue;
      out->ticket = J.ticket;
      out->status = J.rc ? J.rc : (J.info.converged ? VFS_OK : VFS_ERR_NOTCONV);
      out->info = J.info;
      out->divmax = J.divmax;
      if (J.rc) ctx->err = J.err;
      J.g->busy = 0;
      ctx->inflight.erase(it);
      return VFS_OK;
    }
    if (ctx->inflight.empty()) return fail(ctx, VFS_ERR_STATE, "no request in flight");
    std::vector<Job*> js;
    for (auto& kv : ctx->inflight) js.push_back(&kv.second->job);
    int moved = 0;
    bool done = false;
    for (Job* J : js) {
      moved += job_advance_any(ctx, *J);
      done = done || J->phase == J_DONE;
    }
    if (done) continue;
    if (!wait) return VFS_ERR_BUSY;
    if (!moved) wait_any(js);
  }
}

int vfs_inflight(vfs_ctx* ctx) { return ctx ? (int)ctx->inflight.size() : 0; }

int vfs_memory(vfs_ctx* ctx, unsigned long long* used, unsigned long long* budget) {
  if (!ctx) return VFS_ERR_ARG;
  if (used) *used = ctx->used;
  if (budget) *budget = ctx->budget;
  return VFS_OK;
}

int vfs_probe_begin(vfs_ctx* ctx, int kernel) {
  if (!ctx) return VFS_ERR_ARG;
  if (kernel != VFS_PROBE_SMOOTH && kernel != VFS_PROBE_APPLY64 && kernel != VFS_PROBE_ALL)
    return fail(ctx, VFS_ERR_ARG, "unknown probe kernel");
  CK(cudaSetDevice(ctx->device));
  if (g_probe.ev.empty()) {
    g_probe.ev.resize(2 * 8192);
    for (auto& e : g_probe.ev) CK(cudaEventCreate(&e));
  }
  g_probe.kind = kernel;
  g_probe.used = 0;
  g_probe.bytes = 0.;
  g_probe.launches = 0;
  g_probe.recs.clear();
  return VFS_OK;
}

int vfs_probe_end(vfs_ctx* ctx, unsigned long long* launches, double* total_ms, double* alg_bytes) {
  if (!ctx) return VFS_ERR_ARG;
  CK(cudaDeviceSynchronize());
  double ms = 0.;
  for (ProbeRec& r : g_probe.recs) {
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, g_probe.ev[r.ev], g_probe.ev[r.ev + 1]));
    r.ms = t;
    ms += t;
  }
  if (launches) *launches = g_probe.launches;
  if (total_ms) *total_ms = ms;
  if (alg_bytes) *alg_bytes = g_probe.bytes;
  g_probe.kind = 0;
  return VFS_OK;
}

int vfs_probe_record(vfs_ctx* ctx, int i, char* name, int name_len, int* level, double* ms, double* alg_bytes) {
  if (!ctx || i < 0 || i >= (int)g_probe.recs.size()) return VFS_ERR_ARG;
  const ProbeRec& r = g_probe.recs[i];
  if (name && name_len > 0) {
    std::strncpy(name, r.name, (size_t)name_len - 1);
    name[name_len - 1] = 0;
  }
  if (level) *level = r.level;
  if (ms) *ms = r.ms;
  if (alg_bytes) *alg_bytes = r.bytes;
  return VFS_OK;
}

int vfs_launch_count(unsigned long long* out) {
  if (!out) return VFS_ERR_ARG;
  *out = g_launches.load();
  return VFS_OK;
}

int vfs_host_register(void* ptr, unsigned long long bytes) {
  if (!ptr || !bytes) return VFS_ERR_ARG;
  return cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault) == cudaSuccess ? VFS_OK : VFS_ERR_CUDA;
}

int vfs_host_unregister(void* ptr) {
  if (!ptr) return VFS_ERR_ARG;
  return cudaHostUnregister(ptr) == cudaSuccess ? VFS_OK : VFS_ERR_CUDA;
}

int vfs_host_alloc(void** ptr, unsigned long long bytes) {
  if (!ptr || !bytes) return VFS_ERR_ARG;
  *ptr = nullptr;
  if (cudaHostAlloc(ptr, (size_t)bytes, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return VFS_ERR_NOMEM;
  }
  return VFS_OK;
}

int vfs_host_free(void* ptr) {
  if (!ptr) return VFS_ERR_ARG;
  return cudaFreeHost(ptr) == cudaSuccess ? VFS_OK : VFS_ERR_CUDA;
}

int vfs_mark(vfs_ctx* ctx, int grid, int slot) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* g = get_grid(ctx, grid);
  if (!g || slot < 0 || slot >= 4096) return fail(ctx, VFS_ERR_ARG, "no such grid or slot out of [0, 4096)");
  if (ctx->marks.empty()) {
    ctx->marks.resize(4096);
    for (auto& e : ctx->marks) CK(cudaEventCreate(&e));
  }
  CK(cudaEventRecord(ctx->marks[slot], g->s));
  return VFS_OK;
}

int vfs_elapsed(vfs_ctx* ctx, int slot_a, int slot_b, double* ms) {
  if (!ctx || !ms || ctx->marks.empty() || slot_a < 0 || slot_b < 0 || slot_a >= 4096 || slot_b >= 4096)
    return fail(ctx, VFS_ERR_ARG, "bad timer slots");
  CK(cudaEventSynchronize(ctx->marks[slot_b]));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, ctx->marks[slot_a], ctx->marks[slot_b]));
  *ms = t;
  return VFS_OK;
}

int vfs_sync(vfs_ctx* ctx) {
  if (!ctx) return VFS_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  CK(cudaDeviceSynchronize());
  return VFS_OK;
}

// ---- test hooks ----
int vfs_get_level_dims(vfs_ctx* ctx, int grid, int level, int dims[3]) {
  if (!ctx || !dims) return VFS_ERR_ARG;
  Grid* g = get_grid(ctx, grid);
  if (!g || level < 0 || level >= g->L) return fail(ctx, VFS_ERR_ARG, "no such grid or level");
  dims[0] = g->lev[level].d.mx;
  dims[1] = g->lev[level].d.my;
  dims[2] = g->lev[level].d.mz;
  return VFS_OK;
}

int vfs_get_metrics(vfs_ctx* ctx, int grid, int level, double* out) {
  if (!ctx || !out) return VFS_ERR_ARG;
  Grid* g = get_grid(ctx, grid);
  if (!g || level < 0 || level >= g->L) return fail(ctx, VFS_ERR_ARG, "no such grid or level");
  if (int r_ = check_idle(ctx, g)) return r_;
  Level& L = g->lev[level];
  CK(cudaMemcpy(out, L.M, MP_TOTAL * L.N * sizeof(double), cudaMemcpyDeviceToHost));
  return VFS_OK;
}

int vfs_get_level_nvert(vfs_ctx* ctx, int grid, int level, double* out) {
  if (!ctx || !out) return VFS_ERR_ARG;
  Grid* g = get_grid(ctx, grid);
  if (!g || level < 0 || level >= g->L) return fail(ctx, VFS_ERR_ARG, "no such grid or level");
  if (int r_ = check_idle(ctx, g)) return r_;
  Level& L = g->lev[level];
  CK(cudaMemcpy(out, L.nvert, L.N * sizeof(double), cudaMemcpyDeviceToHost));
  return VFS_OK;
}

int vfs_get_coef(vfs_ctx* ctx, int grid, int level, int which, double* out) {
  if (!ctx || !out) return VFS_ERR_ARG;
  Grid* g = get_grid(ctx, grid);
  if (!g || level < 0 || level >= g->L) return fail(ctx, VFS_ERR_ARG, "no such grid or level");
  if (int r_ = check_idle(ctx, g)) return r_;
  if (!g->lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs has not run");
  Level& L = g->lev[level];
  if (which == 0) CK(cudaMemcpy(out, L.coef, 19 * L.N * sizeof(double), cudaMemcpyDeviceToHost));
  else if (which == 1) CK(cudaMemcpy(out, L.mcoef, 19 * L.N * sizeof(double), cudaMemcpyDeviceToHost));
  else if (which == 2) {
    std::vector<float> f(19 * L.N);
    CK(cudaMemcpy(f.data(), L.mcoef32, 19 * L.N * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < f.size(); q++) out[q] = f[q];
  } else return fail(ctx, VFS_ERR_ARG, "which must be 0, 1 or 2");
  return VFS_OK;
}

int vfs_get_mg_half(vfs_ctx* ctx, int grid, int level, double* coef, double* lf, double* rw) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* g = get_grid(ctx, grid);
  if (!g || level < 0 || level >= g->L) return fail(ctx, VFS_ERR_ARG, "no such grid or level");
  if (int r_ = check_idle(ctx, g)) return r_;
  if (!g->lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs has not run");
  Level& L = g->lev[level];
  CK(cudaStreamSynchronize(g->s));
  if (coef) {
    const size_t hs = hslot(L.d);
    std::vector<__half> h(19 * hs);
    CK(cudaMemcpy(h.data(), L.hcoef, h.size() * sizeof(__half), cudaMemcpyDeviceToHost));
    for (int m = 0; m < 19; m++)
      for (size_t c = 0; c < L.N; c++) {
        const int i = (int)(c % L.d.mx), j = (int)((c / L.d.mx) % L.d.my), k = (int)(c / ((size_t)L.d.mx * L.d.my));
        coef[(size_t)m * L.N + c] = (double)__half2float(h[(size_t)m * hs + hidx(L.d, i, j, k)]);
      }
  }
  std::vector<float> f(L.N);
  if (lf) {
    CK(cudaMemcpy(f.data(), L.lfh, L.N * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < L.N; q++) lf[q] = f[q];
  }
  if (rw) {
    CK(cudaMemcpy(f.data(), L.rwh, L.N * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < L.N; q++) rw[q] = f[q];
  }
  return VFS_OK;
}

int vfs_apply_op(vfs_ctx* ctx, int grid, int level, int which, const double* x, double* y) {
  if (!ctx || !x || !y) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp || level < 0 || level >= gp->L) return fail(ctx, VFS_ERR_ARG, "no such grid or level");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  if (!g.lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs has not run");
  Level& L = g.lev[level];
  const size_t N = L.N;
  if (which == 0 || which == 1) {
    double *dx, *dy;
    CK(cudaMalloc(&dx, N * 8));
    CK(cudaMalloc(&dy, N * 8));
    CK(cudaMemcpy(dx, x, N * 8, cudaMemcpyHostToDevice));
    CK(cudaMemset(dy, 0, N * 8));
    if (which == 0) {
      OpView<double> A{L.d, L.coef, L.mask, nullptr};
      launch_apply64(A, dx, nullptr, dy, 0);
    } else {
      OpView<double> A{L.d, L.mcoef, L.mask, nullptr};
      launch_apply_mg<double>(A, dx, nullptr, dy, 0);
    }
    cudaError_t e = cudaMemcpy(y, dy, N * 8, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "apply");
  } else if (which == 2) {
    std::vector<float> hx(N), hy(N);
    for (size_t q = 0; q < N; q++) hx[q] = (float)x[q];
    float *dx, *dy;
    CK(cudaMalloc(&dx, N * 4));
    CK(cudaMalloc(&dy, N * 4));
    CK(cudaMemcpy(dx, hx.data(), N * 4, cudaMemcpyHostToDevice));
    CK(cudaMemset(dy, 0, N * 4));
    OpView<float> A{L.d, L.mcoef32, L.mask, nullptr};
    launch_apply_mg<float>(A, dx, nullptr, dy, 0);
    cudaError_t e = cudaMemcpy(hy.data(), dy, N * 4, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "apply");
    for (size_t q = 0; q < N; q++) y[q] = hy[q];
  } else if (which == 3) {
    // the mixed solver's Krylov product: FP64 aj-scaled operator on FP32 x
    std::vector<float> hx(N);
    for (size_t q = 0; q < N; q++) hx[q] = (float)x[q];
    float* dx;
    double* dy;
    CK(cudaMalloc(&dx, N * 4));
    CK(cudaMalloc(&dy, N * 8));
    CK(cudaMemcpy(dx, hx.data(), N * 4, cudaMemcpyHostToDevice));
    CK(cudaMemset(dy, 0, N * 8));
    OpView<double> A{L.d, L.mcoef, L.mask, nullptr};
    launch_apply64_xf(A, dx, nullptr, dy, 0);
    cudaError_t e = cudaMemcpy(y, dy, N * 8, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "apply");
  } else if (which == 4) {
    // the FP32 face form (the general one on levels with i-j or j-k cross
    // terms) applied to x rounded to FP32
    std::vector<float> hx(N), hy(N);
    for (size_t q = 0; q < N; q++) hx[q] = (float)x[q];
    float *dx, *dy;
    CK(cudaMalloc(&dx, N * 4));
    CK(cudaMalloc(&dy, N * 4));
    CK(cudaMemcpy(dx, hx.data(), N * 4, cudaMemcpyHostToDevice));
    CK(cudaMemset(dy, 0, N * 4));
    OpView<float> A = mgview<float>(L, nullptr, false, true);
    launch_apply_face(A, dx, dy, 0);
    cudaError_t e = cudaMemcpy(hy.data(), dy, N * 4, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "apply");
    for (size_t q = 0; q < N; q++) y[q] = hy[q];
  } else return fail(ctx, VFS_ERR_ARG, "which must be 0, 1, 2, 3 or 4");
  return VFS_OK;
}

int vfs_mg_restrict(vfs_ctx* ctx, int grid, int level, const double* x, double* y) {
  if (!ctx || !x || !y) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp || level < 1 || level >= gp->L) return fail(ctx, VFS_ERR_ARG, "no such grid or level");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  Level &F = g.lev[level], &C = g.lev[level - 1];
  double *dx, *dy;
  CK(cudaMalloc(&dx, F.N * 8));
  CK(cudaMalloc(&dy, C.N * 8));
  CK(cudaMemcpy(dx, x, F.N * 8, cudaMemcpyHostToDevice));
  CK(cudaMemset(dy, 0, C.N * 8));
  launch_restrict<double>(F.d, dx, F.nvert, C.d, C.nvert, g.si, g.sj, g.sk, dy, 0);
  cudaError_t e = cudaMemcpy(y, dy, C.N * 8, cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(dy);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "restrict");
  return VFS_OK;
}

int vfs_mg_prolong(vfs_ctx* ctx, int grid, int level, const double* x, double* y) {
  if (!ctx || !x || !y) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp || level < 1 || level >= gp->L) return fail(ctx, VFS_ERR_ARG, "no such grid or level");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  if (!g.lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs has not run");
  Level &F = g.lev[level], &C = g.lev[level - 1];
  double *dx, *dy;
  CK(cudaMalloc(&dx, C.N * 8));
  CK(cudaMalloc(&dy, F.N * 8));
  CK(cudaMemcpy(dx, x, C.N * 8, cudaMemcpyHostToDevice));
  CK(cudaMemset(dy, 0, F.N * 8));
  launch_prolong<double>(F.d, F.pcode, C.d, dx, dy, 0, nullptr, 0);
  cudaError_t e = cudaMemcpy(y, dy, F.N * 8, cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(dy);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "prolong");
  return VFS_OK;
}

int vfs_grid_components(vfs_ctx* ctx, int grid, int* finest, int* coarsest) {
  if (!ctx) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (!gp->lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs must run first");
  if (finest) *finest = gp->ncomp;
  if (coarsest) *coarsest = gp->ncomp_c;
  return VFS_OK;
}

int vfs_debug_tma_drop(int band) {
  smooth_tma_drop(band < 0 ? -1 : band);
  return VFS_OK;
}

int vfs_sweep_damping(const vfs_solve_params* p, int finest, int post, double* w, int n) {
  if (!p || !w || n < 0) return VFS_ERR_ARG;
  if (p->nu1 < 0 || p->nu2 < 0 || p->nu1 > MAXSWEEP || p->nu2 > MAXSWEEP || p->nu1_coarse < -1 ||
      p->nu2_coarse < -1 || p->nu1_coarse > MAXSWEEP || p->nu2_coarse > MAXSWEEP)
    return VFS_ERR_ARG;
  if (p->smoother != VFS_SMOOTH_JACOBI && p->smoother != VFS_SMOOTH_CHEBYSHEV) return VFS_ERR_ARG;
  if (p->smoother == VFS_SMOOTH_CHEBYSHEV && !(p->cheb_hi > 0. && p->cheb_hi <= 4. && p->cheb_ratio > 1.))
    return VFS_ERR_ARG;
  const MGCfg c = mgcfg(*p, 1);
  const int l = finest ? 1 : 0;
  if (n != (post ? c.post(l) : c.pre(l))) return VFS_ERR_ARG;
  for (int q = 0; q < n; q++) w[q] = c.w(l, post ? 1 : 0, q);
  return VFS_OK;
}

int vfs_mg_smooth(vfs_ctx* ctx, int grid, int level, const double* b, double* x, double omega) {
  if (!ctx || !x || !b) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp || level < 0 || level >= gp->L) return fail(ctx, VFS_ERR_ARG, "no such grid or level");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  if (!g.lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs has not run");
  Level& L = g.lev[level];
  double *db, *dx, *dy;
  CK(cudaMalloc(&db, L.N * 8));
  CK(cudaMalloc(&dx, L.N * 8));
  CK(cudaMalloc(&dy, L.N * 8));
  CK(cudaMemcpy(db, b, L.N * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dx, x, L.N * 8, cudaMemcpyHostToDevice));
  CK(cudaMemset(dy, 0, L.N * 8));
  OpView<double> A{L.d, L.mcoef, L.mask, nullptr};
  launch_smooth<double>(A, L.lf64, dx, db, dy, omega, 0);
  cudaError_t e = cudaMemcpy(x, dy, L.N * 8, cudaMemcpyDeviceToHost);
  cudaFree(db);
  cudaFree(dx);
  cudaFree(dy);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "smooth");
  return VFS_OK;
}

int vfs_apply_precond(vfs_ctx* ctx, int grid, int precision, const vfs_solve_params* p, const double* v, double* z) {
  if (!ctx || !v || !z || !p) return VFS_ERR_ARG;
  Grid* gp = get_grid(ctx, grid);
  if (!gp) return fail(ctx, VFS_ERR_ARG, "no such grid");
  if (int r_ = check_idle(ctx, gp)) return r_;
  Grid& g = *gp;
  if (!g.lhs) return fail(ctx, VFS_ERR_STATE, "vfs_poisson_lhs has not run");
  if (int r_ = check_params(ctx, p)) return r_;
  const size_t N = ncell(g.d);
  Level& F = g.lev[g.L - 1];
  double* dv;
  CK(cudaMalloc(&dv, N * 8));
  CK(cudaMemcpy(dv, v, N * 8, cudaMemcpyHostToDevice));
  int r;
  if (precision == VFS_MIXED) {
    r = ensure_mg<float>(ctx, g);
    float* dz = nullptr;
    if (!r && cudaMalloc(&dz, N * 4) != cudaSuccess) r = VFS_ERR_NOMEM;
    if (!r) cudaMemsetAsync(dz, 0, N * 4, g.s);
    if (!r) r = precond<float>(ctx, g, *p, dv, dz, F.x32[1], nullptr, g.s, true, true);
    if (!r && p->mg_stage == STAGE_TMA) {
      cudaStreamSynchronize(g.s);
      if (smooth_tma_take_error()) r = fail(ctx, VFS_ERR_CUDA, "tensor-copy sweep: a bounded wait ran out");
    }
    if (!r) {
      std::vector<float> hz(N);
      cudaStreamSynchronize(g.s);
      cudaMemcpy(hz.data(), dz, N * 4, cudaMemcpyDeviceToHost);
      for (size_t q = 0; q < N; q++) z[q] = hz[q];
    }
    cudaFree(dz);
  } else {
    r = ensure_mg<double>(ctx, g);
    double* dz = nullptr;
    if (!r && cudaMalloc(&dz, N * 8) != cudaSuccess) r = VFS_ERR_NOMEM;
    if (!r) cudaMemsetAsync(dz, 0, N * 8, g.s);
    if (!r) r = precond<double>(ctx, g, *p, dv, dz, F.x64[1], nullptr, g.s, true, true);
    if (!r) {
      cudaStreamSynchronize(g.s);
      cudaMemcpy(z, dz, N * 8, cudaMemcpyDeviceToHost);
    }
    cudaFree(dz);
  }
  cudaFree(dv);
  return r;
}

}  // extern "C"
