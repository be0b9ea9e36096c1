// server.cu -- continuous batching of root solves, k scans and maps over
// many plasmas (alps_server_*, declared in include/alps_gb300.h).
//
// Admitted requests are grouped by context.  One host thread drives every
// group: an idle group gathers the frequencies all its requests need next
// (the pending evaluations of their root finders, or a lattice).
//
// * Root-finder evaluations on plasmas without relativistic or closed-form
//   species go into fused rounds: one set of kernels evaluates every ready
//   group, each context with the launch shape of a lone batch of its size,
//   so its sums and results are exactly those of a lone batch.  Two rounds
//   can be in flight, on two streams.
// * Lattices, and the plasmas the fused kernels do not take, run as their
//   own batch on the context's stream (replayed as CUDA graphs).
//
// The thread polls the rounds' and batches' events; as one lands it hands
// every request its slice of the determinants (root_finders.h: the
// reference's secant_osc / secant / rtsec), releases the finished requests,
// lets queued requests on that plasma join, and the groups go out again.  A
// k scan moves its context's k, so it runs alone on its context; the k steps
// of all scans ready for one run together (alps_set_k_many: one nmax launch,
// the tables of all contexts, one synchronisation) on a worker thread, one
// such batch at a time.
// Requests join while their estimated device footprint fits the budget.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <future>
#include <map>
#include <mutex>
#include <unordered_set>
#include <thread>
#include <vector>

#include "alps_internal.cuh"
#include "root_finders.h"

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Active {
  alps_request* rq = nullptr;
  int64_t id = 0;
  double t0 = 0.0;
  size_t bytes = 0;
  int status = ALPS_OK;
  // root finders (POLISH, SCAN)
  std::vector<RootMachine> rm;
  std::vector<int> idx;                 // request root index of each machine
  std::vector<std::vector<cplx>> want;  // pending evaluations per machine
  // SCAN state (om_scan, src/ALPS_fns.f90:2198-2600)
  int it = 0, nt = 0, out_row = 0;
  double kp0 = 0, kz0 = 0, th0 = 0, k0 = 0, kperp = 0, kpar = 0;
  std::vector<char> jump;
  // MAP state: the lattice, the det D of its chunks landed so far
  bool map_done = false;
  std::vector<alps_complex> map_lat, map_D;
  size_t off = 0, cnt = 0;  // slice of the group's batch in flight
};

// A map's lattice goes to the device in chunks of this many frequencies,
// one batch each: between two chunks the server launches the other
// requests' rounds, so a large map holds the GPU for a chunk's time, not
// its own.  A lattice of at most this size is one batch, as alps_map runs
// it.
constexpr size_t MAP_CHUNK = 2048;

// The requests admitted on one context.
struct Group {
  alps_ctx* ctx = nullptr;
  std::vector<Active*> members;
  // IN_FLIGHT: a batch on the context's stream; FUSED: in a fused round
  enum { IDLE, IN_FLIGHT, FUSED, STEPPING } state = IDLE;
  std::vector<alps_complex> bom, bD;
  bool has_scan() const {
    for (Active* a : members)
      if (a->rq->kind == ALPS_REQ_SCAN) return true;
    return false;
  }
};

// device bytes of a batch of n frequencies on context c (the per-batch
// buffers of launch_disp_batch plus the staging)
size_t batch_bytes(const alps_ctx* c, size_t n) {
  int S = c->sys.nspec, maxn = 0, rc = 1, relcap = 0;
  for (int s = 0; s < S; ++s) {
    maxn = std::max(maxn, c->spec[s].nmax);
    rc = std::max(rc, c->spec[s].rcap);
    if (c->spec[s].sp.relat) relcap = std::max(relcap, c->spec[s].nmax + 1);
  }
  size_t per = 32 + (size_t)S * ((size_t)(maxn + 1) * 6 * 16 + (size_t)rc * (6 * 16 + 4) + 4 +
                                 (size_t)relcap * 12 * REL_RB * 16 + 24 * 16);
  return n * per;
}

}  // namespace

extern "C" {

// Device memory a context holds: its tables (grids, derivatives, fits,
// Bessel tables, reduced vectors, moments, relativistic and closed-form
// tables) and its batch buffers.
size_t ctx_device_bytes(const alps_ctx* c) {
  const size_t N = c->sys.nperp, M = c->sys.npar, d = sizeof(double);
  size_t b = 0;
  for (const SpeciesHost& S : c->spec) {
    size_t nm = S.nmax + 1;
    if (S.sp.use_bM) {
      b += ((size_t)std::max(S.sp.bM_nmaxs, 0) + 2) * d + (N + 1) * 5 * d;
      continue;
    }
    b += (N + 1 + M + 1) * d + 3 * (N + 1) * (M + 1) * d + (N - 1) * 2 * (M - 1) * d;  // grid, f0, g1, g2, G
    b += (N + 1) * 5 * 4 * d + (N + 1) * 16 * d;                                          // fit, fit_aux
    b += (nm + 2) * (N + 1) * d + 3 * nm * (N - 1) * d + 3 * nm * 2 * (M - 1) * d;       // bessel, Rw, A
    b += nm * (M - 1) * 12 * (d + 16) + (M - 1) * ALPS_KFAR * d + nm * ALPS_KFAR * 12 * (d + 16);  // V, X, mom (+pairs, base tables)
    b += nm * 66 * d;                                                                      // lmom (+pairs)
    if (S.sp.relat) {
      size_t nf = (size_t)(c->sys.ngamma + 1) * (c->sys.npparbar + 1);
      b += 3 * nf * d + (nm + 1) * nf * d + (c->sys.ngamma + 1) * 8;
    }
  }
  b += c->batch_cap * 2 * sizeof(double2) + c->ext_cap * sizeof(double2);
  b += (c->part_cap + c->low_cap + c->items_cap + c->rel_cap + c->bm_cap) * sizeof(double2);
  return b;
}

}  // extern "C"

namespace {

// Sets up a newly admitted request: root finders of a polish, first row of
// a scan (om_scan :2318-2331; a map needs nothing).
void start_request(Active* a) {
  alps_request* rq = a->rq;
  alps_ctx* c = rq->ctx;
  rq->rounds = 0;
  if (rq->kind == ALPS_REQ_POLISH) {
    a->rm.resize(rq->n);
    a->want.resize(rq->n);
    a->idx.resize(rq->n);
    for (int r = 0; r < rq->n; ++r) {
      a->idx[r] = r;
      a->want[r] = a->rm[r].start(&c->sys, c->sys.secant_method, cplx(rq->om[r].re, rq->om[r].im), rq->om_rtol);
    }
    return;
  }
  if (rq->kind == ALPS_REQ_MAP) return;
  const alps_scan_def& sc = rq->scan;
  a->nt = sc.n_out * sc.n_res;
  a->kp0 = a->kperp = c->kperp;
  a->kz0 = a->kpar = c->kpar;
  a->th0 = std::atan(a->kp0 / a->kz0);
  a->k0 = std::sqrt(a->kp0 * a->kp0 + a->kz0 * a->kz0);
  a->jump.assign(rq->n, 1);
  for (int r = 0; r < rq->n; ++r) {
    double* row = rq->scan_rows + (size_t)r * 4;
    row[0] = a->kperp;
    row[1] = a->kpar;
    row[2] = rq->om[r].re;
    row[3] = rq->om[r].im;
  }
  a->out_row = 1;
  a->it = 0;
}

bool evals_pending(const Active* a) {
  for (auto& w : a->want)
    if (!w.empty()) return true;
  return false;
}

// The next k step of a scan, in two parts around the k change:
// scan_step_pre records the step just polished (om_scan :2540-2580) and
// moves the request's k (false when the scan is over); scan_step_post,
// after the context's alps_set_k, starts root finders for the roots still
// followed.  They touch only this request.
bool scan_step_pre(Active* a) {
  alps_request* rq = a->rq;
  alps_ctx* c = rq->ctx;
  if (!a->rm.empty()) {
    for (size_t q = 0; q < a->rm.size(); ++q) {
      int r = a->idx[q];
      cplx o = a->rm[q].root();
      rq->om[r] = alps_complex{o.real(), o.imag()};
      double re = o.real();
      if (std::fabs(re) >= 1.79769313486231571e308 || re != re) a->jump[r] = 0;
      for (int imm = 0; imm < r; ++imm)
        if (std::hypot(rq->om[r].re - rq->om[imm].re, rq->om[r].im - rq->om[imm].im) < c->sys.D_gap) {
          rq->om[r] = alps_complex{0.0, 0.0};
          a->jump[r] = 0;
        }
      if (a->it % rq->scan.n_res == 0) {
        double* row = rq->scan_rows + ((size_t)a->out_row * rq->n + r) * 4;
        row[0] = a->kperp;
        row[1] = a->kpar;
        row[2] = rq->om[r].re;
        row[3] = rq->om[r].im;
      }
    }
    if (a->it % rq->scan.n_res == 0) ++a->out_row;
    a->rm.clear();
    a->want.clear();
    a->idx.clear();
  }
  a->it += 1;
  if (a->it > a->nt) return false;
  scan_k(rq->scan, a->it, a->kp0, a->kz0, a->th0, a->k0, a->kperp, a->kpar);
  return true;
}

void scan_step_post(Active* a, int st) {
  alps_request* rq = a->rq;
  alps_ctx* c = rq->ctx;
  if (st) {
    a->status = st;
    return;
  }
  bool any = false;
  for (int r = 0; r < rq->n; ++r) any = any || a->jump[r];
  if (!any) {
    a->status = ALPS_E_ROOTS_DIVERGED;
    return;
  }
  for (int r = 0; r < rq->n; ++r) {
    if (!a->jump[r]) continue;
    a->idx.push_back(r);
    a->rm.emplace_back();
    a->want.push_back(
        a->rm.back().start(&c->sys, c->sys.secant_method, cplx(rq->om[r].re, rq->om[r].im), rq->om_rtol));
  }
}

// The k steps of every scan in the list on the device together: the output
// of the steps just polished, one alps_set_k_many over the scans that move
// on, the root finders of the new steps.  Runs on a worker thread; touches
// only these requests and their contexts (each owned by its scan).
void scan_steps(std::vector<Active*> list) {
  std::vector<alps_ctx*> ctx;
  std::vector<double> kp, kz;
  std::vector<Active*> moving;
  for (Active* a : list)
    if (scan_step_pre(a)) {
      moving.push_back(a);
      ctx.push_back(a->rq->ctx);
      kp.push_back(a->kperp);
      kz.push_back(a->kpar);
    }
  std::vector<int> st(moving.size(), ALPS_OK);
  if (!moving.empty()) {
    int rc = alps_set_k_many(ctx.data(), (int)ctx.size(), kp.data(), kz.data(), st.data());
    if (rc)
      for (size_t k = 0; k < st.size(); ++k)
        if (!st[k]) st[k] = rc;
  }
  for (size_t k = 0; k < moving.size(); ++k) scan_step_post(moving[k], st[k]);
}

// True once the request has nothing left to do.
bool request_done(const Active* a) {
  const alps_request* rq = a->rq;
  if (a->status != ALPS_OK) return true;
  if (rq->kind == ALPS_REQ_MAP) return a->map_done;
  if (rq->kind == ALPS_REQ_SCAN) return a->it > a->nt;
  return !evals_pending(a);
}

// Upload of the staged frequencies, the batch kernels, download of det D
// and of the error flags, on the context's stream.
int enqueue_batch(alps_ctx* c, int n) {
  ALPS_CUDA_TRY(cudaMemcpyAsync(c->d_om, c->h_pinned, (size_t)n * sizeof(double2), cudaMemcpyHostToDevice, c->stream));
  int st = launch_disp_batch(c, n, c->d_om, c->d_D, nullptr, c->stream);
  if (st) return st;
  ALPS_CUDA_TRY(
      cudaMemcpyAsync(c->h_pinned + n, c->d_D, (size_t)n * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
  ALPS_CUDA_TRY(cudaMemcpyAsync(c->h_flag, c->d_flags, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  return ALPS_OK;
}

// A root finder needs one batch per iteration, each a few frequencies: the
// host cost of its ten or so calls dominates.  After one uncaptured batch of
// a size has run at the context's current state (so every buffer is sized),
// the next one is captured into a CUDA graph and later batches of that size
// replay it with a single launch until the plasma, k, precision or a buffer
// address changes (alps_ctx::gen).
int run_batch(alps_ctx* c, int n) {
  // a graph holds the launch shapes of its capture: the autotuner's epoch
  // is part of its key
  const uint64_t gk = c->gen ^ (tune_epoch() << 40);
  if (!c->profiling) {
    auto it = c->graphs.find(n);
    if (it != c->graphs.end() && it->second.first != gk) {
      cudaGraphExecDestroy(it->second.second);
      c->graphs.erase(it);
      it = c->graphs.end();
    }
    if (it != c->graphs.end()) {
      ALPS_CUDA_TRY(cudaGraphLaunch(it->second.second, c->stream));
      c->stats.graph_replays++;
      return ALPS_OK;
    }
    auto seen = c->graph_seen.find(n);
    if (seen != c->graph_seen.end() && seen->second == gk) {
      const uint64_t gen0 = c->gen;
      cudaGraph_t graph = nullptr;
      bool launched = false;
      if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        int st = enqueue_batch(c, n);
        cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
        cudaGraphExec_t exec = nullptr;
        if (!st && e == cudaSuccess && graph && c->gen == gen0 &&
            cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
          c->graphs[n] = {gk, exec};
          launched = cudaGraphLaunch(exec, c->stream) == cudaSuccess;
          if (launched) c->stats.graph_captures++;
        }
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();  // a refused capture falls back to plain launches
      }
      if (launched) return ALPS_OK;
    }
  }
  int st = enqueue_batch(c, n);
  if (st) return st;
  c->graph_seen[n] = gk;
  return ALPS_OK;
}

// The next evaluations of every request of the group, into g.bom (each
// request's slice at a->off, a->cnt).
void gather_group(Group& g) {
  g.bom.clear();
  for (Active* a : g.members) {
    a->off = g.bom.size();
    if (a->status == ALPS_OK) {
      if (a->rq->kind == ALPS_REQ_MAP) {
        if (!a->map_done) {
          if (a->map_lat.empty()) map_lattice(&a->rq->map, a->map_lat);
          const size_t n0 = a->map_D.size(), n1 = std::min(a->map_lat.size(), n0 + MAP_CHUNK);
          g.bom.insert(g.bom.end(), a->map_lat.begin() + n0, a->map_lat.begin() + n1);
        }
      } else {
        for (auto& w : a->want)
          for (auto& o : w) g.bom.push_back(alps_complex{o.real(), o.imag()});
      }
    }
    a->cnt = g.bom.size() - a->off;
    if (a->cnt) a->rq->rounds += 1;
  }
}

// True when the group's next batch holds a lattice (it then runs on the
// context's own stream, not in a fused round).
bool wants_map(const Group& g) {
  for (const Active* a : g.members)
    if (a->status == ALPS_OK && a->rq->kind == ALPS_REQ_MAP && !a->map_done) return true;
  return false;
}

bool wants_evals(const Group& g) {
  for (const Active* a : g.members)
    if (a->status == ALPS_OK && a->rq->kind != ALPS_REQ_MAP && evals_pending(a)) return true;
  return false;
}

// One batch with the next evaluations of every request of the group, on
// the group's context stream; nothing launched when no request needs any.
int launch_group(Group& g) {
  gather_group(g);
  int n = (int)g.bom.size();
  g.bD.resize(n);
  if (n == 0) return ALPS_OK;
  alps_ctx* c = g.ctx;
  int st = ctx_ensure_batch(c, n, false);
  if (st) return st;
  std::memcpy(c->h_pinned, g.bom.data(), (size_t)n * sizeof(double2));
  if ((st = run_batch(c, n))) return st;
  ALPS_CUDA_TRY(cudaEventRecord(c->ev_done, c->stream));
  g.state = Group::IN_FLIGHT;
  return ALPS_OK;
}

// Hands every request its slice of a landed batch: det D of the group's
// frequencies and the batch's error flags.
void land_slice(Group& g, const alps_complex* batchD, int f) {
  for (Active* a : g.members) {
    if (!a->cnt) continue;
    if (f) {
      a->status = (f & 2) ? ALPS_E_SUBLUMINAL : ALPS_E_INVALID;
      continue;
    }
    const alps_complex* D = batchD + a->off;
    if (a->rq->kind == ALPS_REQ_MAP) {
      a->map_D.insert(a->map_D.end(), D, D + a->cnt);
      if (a->map_D.size() >= a->map_lat.size()) {
        map_finish((int)a->map_D.size(), a->map_D.data(), a->rq->map_cal, a->rq->map_val);
        a->map_done = true;
        std::vector<alps_complex>().swap(a->map_lat);
        std::vector<alps_complex>().swap(a->map_D);
      }
      continue;
    }
    size_t k = 0;
    std::vector<cplx> got;
    for (size_t q = 0; q < a->rm.size(); ++q) {
      if (a->want[q].empty()) continue;
      got.clear();
      for (size_t w = 0; w < a->want[q].size(); ++w, ++k) got.push_back(cplx(D[k].re, D[k].im));
      a->want[q] = a->rm[q].step(got);
    }
  }
}

void land_group(Group& g) {
  alps_ctx* c = g.ctx;
  int n = (int)g.bom.size();
  std::memcpy(g.bD.data(), c->h_pinned + n, (size_t)n * sizeof(double2));
  land_slice(g, g.bD.data(), *c->h_flag);
}

// A fused round: the next evaluations of many groups (root finders on
// fusable contexts) in one set of kernels on the round's stream.
struct Round {
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;   // the round's last copy (timing: the round's device span from ev0)
  cudaEvent_t ev0 = nullptr;  // before the round's first copy
  size_t jobs = 0;
  MultiScratch* scratch = nullptr;
  double2* d_om = nullptr;
  double2* d_D = nullptr;
  alps_complex* h_om = nullptr;  // pinned
  alps_complex* h_D = nullptr;   // pinned
  size_t cap = 0;
  int* d_flags = nullptr;
  int* h_flags = nullptr;  // pinned
  size_t fcap = 0;
  std::vector<Group*> groups;
  std::vector<size_t> off;  // first frequency of each group
  bool busy = false;

  ~Round() {
    if (st) cudaStreamSynchronize(st);
    multi_scratch_free(scratch);
    cudaFree(d_om);
    cudaFree(d_D);
    cudaFreeHost(h_om);
    cudaFreeHost(h_D);
    cudaFree(d_flags);
    cudaFreeHost(h_flags);
    if (ev) cudaEventDestroy(ev);
    if (ev0) cudaEventDestroy(ev0);
    if (st) cudaStreamDestroy(st);
  }

  int reserve(size_t n, size_t nj) {
    if (!st) {
      // root-finding rounds are latency-bound: their stream has the
      // device's highest priority, so the block scheduler serves them ahead
      // of map lattices (context streams, default priority) already running
      int lo = 0, hi = 0;
      ALPS_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
      ALPS_CUDA_TRY(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, hi));
      ALPS_CUDA_TRY(cudaEventCreate(&ev));
      ALPS_CUDA_TRY(cudaEventCreate(&ev0));
    }
    if (n > cap) {
      const size_t c2 = std::max(n, 2 * cap);
      cudaFree(d_om);
      cudaFree(d_D);
      cudaFreeHost(h_om);
      cudaFreeHost(h_D);
      d_om = d_D = nullptr;
      h_om = h_D = nullptr;
      cap = 0;
      ALPS_CUDA_TRY(cudaMalloc(&d_om, c2 * sizeof(double2)));
      ALPS_CUDA_TRY(cudaMalloc(&d_D, c2 * sizeof(double2)));
      ALPS_CUDA_TRY(cudaMallocHost(&h_om, c2 * sizeof(alps_complex)));
      ALPS_CUDA_TRY(cudaMallocHost(&h_D, c2 * sizeof(alps_complex)));
      cap = c2;
    }
    if (nj > fcap) {
      cudaFree(d_flags);
      cudaFreeHost(h_flags);
      d_flags = nullptr;
      h_flags = nullptr;
      fcap = 0;
      ALPS_CUDA_TRY(cudaMalloc(&d_flags, nj * sizeof(int)));
      ALPS_CUDA_TRY(cudaMallocHost(&h_flags, nj * sizeof(int)));
      fcap = nj;
    }
    return ALPS_OK;
  }

  // gathers and launches the next evaluations of the ready groups
  int launch(const std::vector<Group*>& ready) {
    groups.clear();
    off.clear();
    std::vector<alps_ctx*> ctx;
    std::vector<int> ns;
    size_t n = 0;
    for (Group* g : ready) {
      gather_group(*g);
      if (g->bom.empty()) continue;
      groups.push_back(g);
      off.push_back(n);
      ctx.push_back(g->ctx);
      ns.push_back((int)g->bom.size());
      n += g->bom.size();
    }
    if (groups.empty()) return ALPS_OK;
    int st_ = reserve(n, groups.size());
    if (st_) return st_;
    for (size_t j = 0; j < groups.size(); ++j)
      std::memcpy(h_om + off[j], groups[j]->bom.data(), groups[j]->bom.size() * sizeof(alps_complex));
    jobs = groups.size();
    ALPS_CUDA_TRY(cudaEventRecord(ev0, st));
    ALPS_CUDA_TRY(cudaMemcpyAsync(d_om, h_om, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    if ((st_ = launch_disp_multi(ctx.data(), ns.data(), (int)ctx.size(), d_om, d_D, d_flags, &scratch, st)))
      return st_;
    ALPS_CUDA_TRY(cudaMemcpyAsync(h_D, d_D, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    ALPS_CUDA_TRY(cudaMemcpyAsync(h_flags, d_flags, groups.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
    ALPS_CUDA_TRY(cudaEventRecord(ev, st));
    for (Group* g : groups) g->state = Group::FUSED;
    busy = true;
    return ALPS_OK;
  }

  void land() {
    for (size_t j = 0; j < groups.size(); ++j) {
      land_slice(*groups[j], h_D + off[j], h_flags[j]);
      groups[j]->state = Group::IDLE;
    }
    groups.clear();
    busy = false;
  }
};

}  // namespace


struct alps_server {
  size_t budget = 0;
  int max_active = 256;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::pair<int64_t, alps_request*>> queue;
  std::map<int64_t, alps_request*> pending;  // submitted, not finished
  std::map<int64_t, int> finished;           // id -> status
  std::map<int64_t, double> t_submit;
  int64_t next_id = 1;
  bool stop = false;
  std::thread th;
  // statistics
  int64_t batches = 0;
  int peak_active = 0;
  size_t peak_bytes = 0;
  alps_server_profile prof = {};  // written by the server thread under prof_mu
  std::mutex prof_mu;

  void run();
  void finish(Active* a);
};

void alps_server::finish(Active* a) {
  alps_request* rq = a->rq;
  if (rq->kind == ALPS_REQ_POLISH && a->status == ALPS_OK)
    for (size_t k = 0; k < a->rm.size(); ++k) {
      cplx o = a->rm[k].root();
      rq->om[k] = alps_complex{o.real(), o.imag()};
      if (rq->iters) rq->iters[k] = a->rm[k].iters();
      if (rq->converged) rq->converged[k] = a->rm[k].converged() ? 1 : 0;
    }
  rq->status = a->status;
  rq->latency_ms = now_ms() - a->t0;
  std::lock_guard<std::mutex> lk(mu);
  finished[a->id] = a->status;
  pending.erase(a->id);
  t_submit.erase(a->id);
  cv_done.notify_all();
}

void alps_server::run() {
  std::map<alps_ctx*, Group> groups;
  Round rounds[2];  // fused rounds in flight at once
  size_t in_use = 0;
  int n_active = 0;
  bool step_busy = false;         // a batch of scan k steps is on its worker thread
  std::future<void> step_future;
  std::chrono::steady_clock::time_point t_step;
  for (;;) {
    const auto t_loop = std::chrono::steady_clock::now();
    {
      std::unique_lock<std::mutex> lk(mu);
      // admission, in submission order: a request joins its context's group
      // while the group is between batches, holds no scan, and (for a scan)
      // is empty, and while the footprint fits the budget
      std::unordered_set<alps_ctx*> blocked;  // contexts whose earlier request waits
      for (auto itq = queue.begin(); itq != queue.end() && n_active < max_active;) {
        alps_request* rq = itq->second;
        auto gi = groups.find(rq->ctx);
        bool ok = blocked.count(rq->ctx) == 0;
        if (ok && gi != groups.end()) {
          Group& g = gi->second;
          ok = g.state == Group::IDLE && !g.has_scan() && (rq->kind != ALPS_REQ_SCAN || g.members.empty());
        }
        size_t need = 0;
        if (ok) {
          const size_t nb =
              (rq->kind == ALPS_REQ_MAP) ? std::min((size_t)rq->map.nr * rq->map.ni, MAP_CHUNK)
                                         : (size_t)2 * std::max(rq->n, 1);
          need = batch_bytes(rq->ctx, nb) + (gi == groups.end() ? ctx_device_bytes(rq->ctx) : 0);
        }
        if (!ok || (in_use + need > budget && n_active > 0)) {
          // keep the context's order: later requests on it wait too
          blocked.insert(rq->ctx);
          ++itq;
          continue;
        }
        Group& g = groups[rq->ctx];
        g.ctx = rq->ctx;
        Active* a = new Active();
        a->rq = rq;
        a->id = itq->first;
        a->t0 = t_submit[itq->first];
        a->bytes = need;
        in_use += need;
        ++n_active;
        g.members.push_back(a);
        start_request(a);
        itq = queue.erase(itq);
      }
      peak_active = std::max(peak_active, n_active);
      peak_bytes = std::max(peak_bytes, in_use);
      {
        std::lock_guard<std::mutex> pl(prof_mu);
        prof.admit_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_loop).count();
      }
      if (groups.empty()) {
        if (stop && queue.empty()) return;
        cv_work.wait(lk);
        continue;
      }
    }
    bool progressed = false;
    for (Round& R : rounds) {
      if (!R.busy) continue;
      cudaError_t q = cudaEventQuery(R.ev);
      if (q == cudaErrorNotReady) continue;
      progressed = true;
      if (q == cudaSuccess) {
        float ms = 0.0f;
        const auto t0 = std::chrono::steady_clock::now();
        R.land();
        std::lock_guard<std::mutex> pl(prof_mu);
        if (cudaEventElapsedTime(&ms, R.ev0, R.ev) == cudaSuccess) prof.round_gpu_ms += ms;
        prof.land_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      } else {
        alps_set_last_cuda_error(q, "cudaEventQuery", __FILE__, __LINE__);
        for (Group* g : R.groups) {
          for (Active* a : g->members) a->status = ALPS_E_CUDA;
          g->state = Group::IDLE;
        }
        R.groups.clear();
        R.busy = false;
      }
    }
    // the batch of scan k steps in flight: when it has landed its groups go
    // back to IDLE in the loop below, and the scans ready now form the next
    bool step_done = false;
    if (step_busy && step_future.wait_for(std::chrono::seconds(0)) == std::future_status::ready) {
      step_future.get();
      step_busy = false;
      step_done = true;
      std::lock_guard<std::mutex> pl(prof_mu);
      prof.step_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_step).count();
    }
    std::vector<Group*> step_groups;
    std::vector<Active*> step_list;
    std::vector<Group*> ready;  // groups whose next batch can join a fused round
    const auto t_groups = std::chrono::steady_clock::now();
    for (auto gi = groups.begin(); gi != groups.end();) {
      Group& g = gi->second;
      if (g.state == Group::STEPPING) {
        if (step_done) {
          g.state = Group::IDLE;
          progressed = true;
        }
      } else if (g.state == Group::IN_FLIGHT) {
        cudaError_t q = cudaEventQuery(g.ctx->ev_done);
        if (q != cudaErrorNotReady) {
          g.state = Group::IDLE;
          progressed = true;
          if (q == cudaSuccess) {
            land_group(g);
          } else {
            alps_set_last_cuda_error(q, "cudaEventQuery", __FILE__, __LINE__);
            for (Active* a : g.members) a->status = ALPS_E_CUDA;
          }
        }
      }
      if (g.state == Group::IDLE) {
        // release the finished requests of the group
        for (size_t q = 0; q < g.members.size();) {
          Active* a = g.members[q];
          if (request_done(a)) {
            finish(a);
            in_use -= a->bytes;
            --n_active;
            delete a;
            g.members.erase(g.members.begin() + q);
            progressed = true;
          } else {
            ++q;
          }
        }
        // a scan whose step is polished moves to its next k off this thread
        Active* sc = nullptr;
        for (Active* a : g.members)
          if (a->rq->kind == ALPS_REQ_SCAN && !evals_pending(a)) sc = a;
        if (sc) {
          // waits for the next step batch (one in flight at a time)
          if (!step_busy) {
            g.state = Group::STEPPING;
            step_groups.push_back(&g);
            step_list.push_back(sc);
          }
        } else if (!g.members.empty()) {
          if (!wants_map(g) && wants_evals(g) && ctx_fusable(g.ctx)) {
            ready.push_back(&g);
          } else {
            int st = launch_group(g);
            if (st)
              for (Active* a : g.members) a->status = st;
            if (g.state == Group::IN_FLIGHT) {
              ++batches;
              std::lock_guard<std::mutex> pl(prof_mu);
              prof.group_batches++;
            }
            progressed = true;
          }
        }
      }
      if (g.state == Group::IDLE && g.members.empty())
        gi = groups.erase(gi);
      else
        ++gi;
    }
    {
      std::lock_guard<std::mutex> pl(prof_mu);
      prof.groups_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_groups).count();
    }
    if (!step_list.empty()) {
      {
        std::lock_guard<std::mutex> pl(prof_mu);
        prof.scan_step_batches++;
        prof.scan_steps += (int64_t)step_list.size();
      }
      t_step = std::chrono::steady_clock::now();
      step_future = std::async(std::launch::async, scan_steps, step_list);
      step_busy = true;
      progressed = true;
    }
    if (!ready.empty()) {
      // with both round slots free the ready groups split in two, so that
      // two rounds stay in flight and one's tail overlaps the other's work
      std::vector<Round*> free_rounds;
      for (Round& R : rounds)
        if (!R.busy) free_rounds.push_back(&R);
      const size_t parts = std::min(free_rounds.size(), ready.size());
      for (size_t k = 0; k < parts; ++k) {
        std::vector<Group*> share(ready.begin() + ready.size() * k / parts,
                                  ready.begin() + ready.size() * (k + 1) / parts);
        Round& R = *free_rounds[k];
        const auto t0 = std::chrono::steady_clock::now();
        int st = R.launch(share);
        {
          std::lock_guard<std::mutex> pl(prof_mu);
          prof.round_launch_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        }
        if (st)
          for (Group* g : share)
            for (Active* a : g->members) a->status = st;
        batches += (int64_t)R.groups.size();
        if (R.busy) {
          std::lock_guard<std::mutex> pl(prof_mu);
          prof.rounds++;
          prof.round_jobs += (int64_t)R.jobs;
        }
        progressed = true;
      }
    }
    if (progressed) {
      std::lock_guard<std::mutex> pl(prof_mu);
      prof.loop_busy_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_loop).count();
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(5));
  }
}

extern "C" {

int alps_server_create(size_t hbm_budget, int max_active, alps_server** out) {
  if (!out) return ALPS_E_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return ALPS_E_NO_DEVICE;
  alps_server* s = new alps_server();
  if (hbm_budget == 0) {
    size_t fr = 0, tot = 0;
    ALPS_CUDA_TRY(cudaMemGetInfo(&fr, &tot));
    hbm_budget = (size_t)(0.9 * (double)fr);
  }
  s->budget = hbm_budget;
  s->max_active = max_active > 0 ? max_active : 256;
  s->th = std::thread([s]() { s->run(); });
  *out = s;
  return ALPS_OK;
}

void alps_server_destroy(alps_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
  }
  if (s->th.joinable()) s->th.join();
  delete s;
}

int alps_server_submit(alps_server* s, alps_request* rq, int64_t* id) {
  if (!s || !rq || !rq->ctx || !rq->ctx->kset) return ALPS_E_INVALID;
  if (rq->kind == ALPS_REQ_POLISH && (rq->n < 0 || (rq->n > 0 && !rq->om))) return ALPS_E_INVALID;
  if (rq->kind == ALPS_REQ_MAP && (rq->map.nr < 1 || rq->map.ni < 1)) return ALPS_E_INVALID;
  if (rq->kind == ALPS_REQ_SCAN &&
      (rq->n < 1 || !rq->om || !rq->scan_rows || rq->scan.n_out < 0 || rq->scan.n_res < 1 || rq->scan.type_s < 0 ||
       rq->scan.type_s > 4))
    return ALPS_E_INVALID;
  if (rq->kind < ALPS_REQ_POLISH || rq->kind > ALPS_REQ_SCAN) return ALPS_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return ALPS_E_INVALID;
  rq->status = ALPS_OK;
  rq->latency_ms = 0.0;
  int64_t k = s->next_id++;
  s->t_submit[k] = now_ms();
  s->queue.push_back({k, rq});
  s->pending[k] = rq;
  if (id) *id = k;
  s->cv_work.notify_all();
  return ALPS_OK;
}

int alps_server_poll(alps_server* s, int64_t id, int* done) {
  if (!s || !done) return ALPS_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->finished.count(id)) {
    *done = 1;
    return ALPS_OK;
  }
  if (!s->pending.count(id)) return ALPS_E_INVALID;
  *done = 0;
  return ALPS_OK;
}

int alps_server_wait(alps_server* s, int64_t id) {
  if (!s) return ALPS_E_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  if (!s->finished.count(id) && !s->pending.count(id)) return ALPS_E_INVALID;
  s->cv_done.wait(lk, [&]() { return s->finished.count(id) > 0; });
  return s->finished[id];
}

int alps_server_get_profile(alps_server* s, alps_server_profile* out) {
  if (!s || !out) return ALPS_E_INVALID;
  std::lock_guard<std::mutex> pl(s->prof_mu);
  *out = s->prof;
  return ALPS_OK;
}

int alps_server_stats(alps_server* s, int64_t* rounds, int* peak_active, size_t* peak_bytes) {
  if (!s) return ALPS_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (rounds) *rounds = s->batches;
  if (peak_active) *peak_active = s->peak_active;
  if (peak_bytes) *peak_bytes = s->peak_bytes;
  return ALPS_OK;
}

}  // extern "C"
