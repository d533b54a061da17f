// sg_batch.cu -- many independent map-making problems at once, and the FFT
// tile-shape autotuner (no reference counterpart: the reference solves one
// problem per run).
//
// sg_solve_batch runs the PCG of every context concurrently: each context
// iterates on its own CUDA stream, one captured graph launch per iteration,
// and a host loop advances each problem as soon as its previous iteration has
// finished (an event per context, no device-wide synchronisation).  Small
// problems, whose kernels cannot fill 152 SMs, then share the GPU, and a
// problem that converges early stops consuming it.
//
// sg_autotune times the noise filter of a context with each compiled tile
// shape for its segment length (FP32: 8192 or 4096 complex points per CTA of
// the cluster) on the context's own timeline, or with the offset-group
// operator one whole operator application, and keeps the faster one; then
// the P^T reduction's team of lanes per pixel (half, the same and twice the
// size chosen from the mean samples per pixel), timed on its own.
#include <cuda_runtime.h>

#include <cstdlib>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "sg_ctx.h"
#include "sg_kernels.h"

extern "C" int sg_tile_shapes(const sg_ctx* c, int* cluster_size, int* pt_lanes_out) {
  if (!c) return SG_ERR_ARG;
  if (!c->have_pointing) return SG_ERR_STATE;
  if (cluster_size) *cluster_size = c->S;
  if (pt_lanes_out) *pt_lanes_out = c->f32 ? c->pt_team() : 32;
  return SG_OK;
}

extern "C" int sg_autotune(sg_ctx* c, int* cluster_size, double* ms) {
  if (!c) return SG_ERR_ARG;
  if (!c->have_pointing) return c->fail(SG_ERR_STATE, "pointing not set");
  for (long long dd = 0; dd < c->ndet; dd++)
    if (!c->have_noise[dd]) return c->fail(SG_ERR_STATE, "noise of detector %lld not set", dd);
  cudaSetDevice(c->desc.device);
  const long long M = c->ns / 2;
  std::vector<int> cand;
  const long long e1 = c->f32 ? 8192 : 4096;
  for (long long emax : {e1, e1 / 2}) {
    const int S = (int)std::max<long long>(1, M / emax);
    const int ncl = c->f32 ? filter_max_clusters<float>(c->logm, S)
                           : filter_max_clusters<double>(c->logm, S);
    if (ncl > 0 && (cand.empty() || cand.back() != S)) cand.push_back(S);
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int S0 = c->S, n0 = c->nclusters;
  int bestS = S0;
  double best = 1e30;
  cudaError_t e = cudaSuccess;
  for (int S : cand) {
    c->S = S;
    c->nclusters = c->f32 ? filter_max_clusters<float>(c->logm, S)
                          : filter_max_clusters<double>(c->logm, S);
    // the offset-group operator runs the spectrum-split filter on its group
    // tiles: time one whole operator application (its slot order follows S)
    if (c->group_mode) e = c->ensure_hmix();
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {  // first launch warms up
      if (rep == 1) e = cudaEventRecord(a, c->st);
      if (e != cudaSuccess) break;
      e = c->grouped()
              ? c->apply_dev(c->x.as<double>(), c->q.as<double>(), true)
              : c->launch_filter(kLoadTod, c->tod.p, c->y.p, c->ntiles, (int)c->nseg, 0);
    }
    if (e == cudaSuccess) e = cudaEventRecord(b, c->st);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float t = 0.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&t, a, b);
    if (e == cudaSuccess && t / 3.0 < best) {
      best = t / 3.0;
      bestS = S;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  c->S = bestS;
  c->nclusters = c->f32 ? filter_max_clusters<float>(c->logm, bestS)
                        : filter_max_clusters<double>(c->logm, bestS);
  if (e == cudaSuccess && (bestS != S0 || c->nclusters != n0)) {
    e = c->chi2p.alloc(sizeof(double) * c->S * c->nclusters);
    c->drop_graphs();  // captured iterations hold the old launch shape
  }
  if (e == cudaSuccess && c->group_mode) e = c->ensure_hmix();  // slot order of the chosen S
  // the P^T reduction tile: lanes per pixel (FP32 only; the FP64 kernel uses
  // a warp per pixel).  It reads the per-group-sample sums the filter left.
  if (e == cudaSuccess && c->f32) {
    const int L0 = pt_lanes(c->ngsamp, c->npix), Lk = c->pt_L;
    int bestL = L0;
    double bestt = 1e30;
    for (int L : {L0 / 2, L0, 2 * L0}) {
      if (L < 1 || L > 32) continue;
      c->pt_L = L;
      cudaEvent_t a2, b2;
      cudaEventCreate(&a2);
      cudaEventCreate(&b2);
      for (int rep = 0; rep < 6 && e == cudaSuccess; rep++) {  // first launch warms up
        if (rep == 1) e = cudaEventRecord(a2, c->st);
        if (e == cudaSuccess) e = c->launch_pt(c->q.as<double>(), true);
      }
      if (e == cudaSuccess) e = cudaEventRecord(b2, c->st);
      if (e == cudaSuccess) e = cudaEventSynchronize(b2);
      float t = 0.f;
      if (e == cudaSuccess) cudaEventElapsedTime(&t, a2, b2);
      cudaEventDestroy(a2);
      cudaEventDestroy(b2);
      if (e == cudaSuccess && t < bestt) {
        bestt = t;
        bestL = L;
      }
    }
    c->pt_L = bestL;
    if (bestL != (Lk > 0 ? Lk : L0)) c->drop_graphs();  // captured iterations hold the old team
  }
  if (e != cudaSuccess) return c->cuda_fail(e, "autotune");
  if (cluster_size) *cluster_size = c->S;
  if (ms) *ms = best;
  return SG_OK;
}

namespace {

struct Job {
  sg_ctx* c = nullptr;
  int pc = 1, iter = 0, fallback = -1;
  bool started = false, pending = false, done = false;
  double var00 = 0.0, crit = 0.0, t_done = 0.0;
  long long launches0 = 0;
  cudaEvent_t ready = nullptr;
};

// enqueue a solve start from x = 0 (r = 0 -> r = b) for precond pc
cudaError_t enqueue_start(sg_ctx* c, int pc) {
  const size_t vb = sizeof(double) * 3 * c->npix;
  cudaError_t e = cudaMemsetAsync(c->x.p, 0, vb, c->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->r.p, 0, vb, c->st);
  CgVecs v = c->vecs(pc == 2 ? 1 : pc);
  if (e == cudaSuccess) e = c->f32 ? cg_init<float>(v, c->st) : cg_init<double>(v, c->st);
  c->launches += 2;
  if (pc == 2) {
    CgVecs v2 = c->vecs(2);
    if (e == cudaSuccess) e = c->learned_z(0);
    if (e == cudaSuccess)
      e = c->f32 ? cg_reinit_d<float>(v2, c->dmap.as<float>(), c->st)
                 : cg_reinit_d<double>(v2, c->dmap.as<double>(), c->st);
    c->launches += 1;
  } else if (e == cudaSuccess) {
    e = c->to_map(c->d.as<double>());
  }
  return e;
}

cudaError_t enqueue_scalars(Job& j) {
  sg_ctx* c = j.c;
  cudaError_t e =
      cudaMemcpyAsync(c->sc_host, c->sc.p, sizeof(CgScalars), cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaEventRecord(j.ready, c->st);
  j.pending = e == cudaSuccess;
  return e;
}

// ---- the whole batch as one graph launch ---------------------------------------
// For every problem: [solve start, WHILE loop of its iterations], independent
// branches of one graph, so the 32 solves are one launch.  The
// captured graph is kept for the same contexts (same captured state, checked
// by each context's graph generation) and dropped when a context goes away.
struct BatchGraph {
  cudaGraphExec_t exec = nullptr;
  std::vector<unsigned long long> gens;
  std::vector<int> pcs, rkinds;
  std::vector<long long> nref, nplain, nstart;
};
std::mutex g_batch_mu;
std::map<std::vector<const sg_ctx*>, BatchGraph> g_batch;

cudaError_t build_batch_graph(std::vector<Job>& jobs, BatchGraph& bg) {
  cudaGraph_t G;
  cudaError_t e = cudaGraphCreate(&G, 0);
  if (e != cudaSuccess) return e;
  const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
  for (size_t i = 0; i < jobs.size() && e == cudaSuccess; i++) {
    sg_ctx* c = jobs[i].c;
    cudaGraph_t cap;
    e = cudaStreamBeginCaptureToGraph(c->st, G, nullptr, nullptr, 0, mode);
    if (e != cudaSuccess) break;
    const long long before = c->launches;
    e = enqueue_start(c, jobs[i].pc);
    bg.nstart[i] = c->launches - before;
    c->launches = before;
    std::vector<cudaGraphNode_t> deps;
    if (e == cudaSuccess) {
      cudaStreamCaptureStatus status;
      const cudaGraphNode_t* d = nullptr;
      size_t nd = 0;
      e = cudaStreamGetCaptureInfo(c->st, &status, nullptr, nullptr, &d, nullptr, &nd);
      if (e == cudaSuccess) deps.assign(d, d + nd);
    }
    cudaError_t e2 = cudaStreamEndCapture(c->st, &cap);
    if (e == cudaSuccess) e = e2;
    cudaGraphNode_t loop;
    if (e == cudaSuccess)
      e = c->add_solve_loop(G, deps.data(), deps.size(), jobs[i].pc, &loop, &bg.nref[i],
                            &bg.nplain[i]);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&bg.exec, G, 0);
  cudaGraphDestroy(G);
  return e;
}

}  // namespace

void forget_batch_graphs(const sg_ctx* c) {
  std::lock_guard<std::mutex> lk(g_batch_mu);
  for (auto it = g_batch.begin(); it != g_batch.end();) {
    bool uses = false;
    for (const sg_ctx* x : it->first) uses |= x == c;
    if (uses) {
      if (it->second.exec) cudaGraphExecDestroy(it->second.exec);
      it = g_batch.erase(it);
    } else {
      ++it;
    }
  }
}

// one graph launch for all problems; false if the batch cannot run this way
static int solve_batch_device(std::vector<Job>& jobs, const sg_solve_opts* o, int maxiter,
                              int refresh_every, sg_report* reports) {
  const int n = (int)jobs.size();
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < n && e == cudaSuccess; i++) {
    sg_ctx* c = jobs[i].c;
    e = c->ensure_loop_buffers(maxiter);  // (may drop captured graphs)
    LoopState ls{0, maxiter, refresh_every, 0, o->stop_crit, 0, 0, jobs[i].pc != 0 ? 1 : 0};
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->loop_state.p, &ls, sizeof(ls), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  }
  if (e != cudaSuccess) return jobs[0].c->cuda_fail(e, "batch loop set-up");
  std::vector<const sg_ctx*> key(n);
  for (int i = 0; i < n; i++) key[i] = jobs[i].c;
  std::lock_guard<std::mutex> lk(g_batch_mu);
  BatchGraph& bg = g_batch[key];
  bool fresh = bg.exec != nullptr;
  for (int i = 0; i < n && fresh; i++)
    fresh = bg.gens[i] == jobs[i].c->graph_gen && bg.pcs[i] == jobs[i].pc &&
            bg.rkinds[i] == jobs[i].c->refresh_kind();
  if (!fresh) {
    if (bg.exec) cudaGraphExecDestroy(bg.exec);
    bg = BatchGraph{};
    bg.nref.assign(n, 0);
    bg.nplain.assign(n, 0);
    bg.nstart.assign(n, 0);
    e = build_batch_graph(jobs, bg);
    if (e != cudaSuccess) {
      if (bg.exec) cudaGraphExecDestroy(bg.exec);
      g_batch.erase(key);
      return jobs[0].c->cuda_fail(e, "batch graph");
    }
    for (int i = 0; i < n; i++) {
      bg.gens.push_back(jobs[i].c->graph_gen);
      bg.pcs.push_back(jobs[i].pc);
      bg.rkinds.push_back(jobs[i].c->refresh_kind());
    }
  }
  sg_ctx* c0 = jobs[0].c;
  const double t0 = now_s();
  e = cudaGraphLaunch(bg.exec, c0->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c0->st);
  const double t1 = now_s();
  if (e != cudaSuccess) return c0->cuda_fail(e, "batch graph launch");
  unsigned long long t_begin = ~0ULL;  // the device clock at the first problem's first iteration
  std::vector<LoopState> states(n);
  for (int i = 0; i < n && e == cudaSuccess; i++) {
    e = cudaMemcpy(&states[i], jobs[i].c->loop_state.p, sizeof(LoopState), cudaMemcpyDeviceToHost);
    if (states[i].iter > 0 && states[i].t_first < t_begin) t_begin = states[i].t_first;
  }
  if (e != cudaSuccess) return c0->cuda_fail(e, "batch results");
  for (int i = 0; i < n; i++) {
    Job& j = jobs[i];
    sg_ctx* c = j.c;
    const LoopState& ls = states[i];
    e = cudaMemcpy(c->sc_host, c->sc.p, sizeof(CgScalars), cudaMemcpyDeviceToHost);
    c->crit_hist.resize(ls.iter);
    if (e == cudaSuccess && ls.iter > 0)
      e = cudaMemcpy(c->crit_hist.data(), c->loop_hist.p, sizeof(double) * ls.iter,
                     cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return c->cuda_fail(e, "batch results");
    j.iter = ls.iter;
    j.var00 = c->sc_host->var00;
    j.crit = c->sc_host->var / j.var00;
    const long long nr = refresh_count(ls.iter, refresh_every, j.pc != 0 ? 1 : 0);
    c->launches += bg.nstart[i] + nr * bg.nref[i] + (ls.iter - nr) * bg.nplain[i] + 2LL * ls.iter;
    if (ls.done == 3 && j.pc == 2 && j.crit > o->stop_crit) {
      // the learned part broke flexible PCG: finish this problem with plain
      // block-Jacobi PCG from its current map, driven from the host
      j.fallback = j.iter;
      j.pc = 1;
      CgVecs v1 = c->vecs(1);
      e = c->apply_dev(c->x.as<double>(), c->r.as<double>(), true);
      if (e == cudaSuccess) e = c->f32 ? cg_init<float>(v1, c->st) : cg_init<double>(v1, c->st);
      if (e == cudaSuccess) e = c->to_map(c->d.as<double>());
      c->launches += 7;
      while (e == cudaSuccess && j.iter < maxiter && j.crit > o->stop_crit) {
        e = c->run_iteration(1, refresh_at(j.iter, refresh_every, 1), true);
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(c->sc_host, c->sc.p, sizeof(CgScalars), cudaMemcpyDeviceToHost, c->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
        if (e != cudaSuccess) break;
        j.crit = c->sc_host->var / j.var00;
        c->crit_hist.push_back(j.crit);
        j.iter++;
        if (c->sc_host->flag) break;
      }
      if (e != cudaSuccess) return c->cuda_fail(e, "batch fallback");
    }
    // device time from the batch's first iteration to this problem's last one
    const double ms = ls.iter > 0 ? (double)(ls.t_last - t_begin) * 1e-6 : 0.0;
    c->have_solution = true;
    if (reports) {
      sg_report& r = reports[i];
      r = sg_report{};
      r.iterations = j.iter;
      r.converged = j.crit <= o->stop_crit;
      r.crit = j.crit;
      r.var00 = j.var00;
      r.solve_seconds = t1 - t0;
      r.iter_per_sec = j.iter / (t1 - t0 > 0 ? t1 - t0 : 1e-30);
      r.device_seconds = ms * 1e-3;
      r.kernel_launches = (long)(c->launches - j.launches0);
      r.breakdown = c->sc_host->flag;
      r.fallback_iter = j.fallback;
    }
  }
  return SG_OK;
}

extern "C" int sg_solve_batch(sg_ctx** ctxs, int n, const sg_solve_opts* o, sg_report* reports) {
  if (!ctxs || n <= 0 || !o) return SG_ERR_ARG;
  if (o->x0) return SG_ERR_ARG;  // every batch solve starts from x = 0
  std::vector<Job> jobs(n);
  for (int i = 0; i < n; i++) {
    sg_ctx* c = ctxs[i];
    if (!c) return SG_ERR_ARG;
    if (!c->have_rhs) return c->fail(SG_ERR_STATE, "call sg_rhs before sg_solve_batch");
    if (o->precond == SG_PRECOND_LEARNED && !c->have_mlp && c->coarse_k == 0)
      return c->fail(SG_ERR_STATE, "no trained network or coarse space");
    cudaSetDevice(c->desc.device);
    int rc = (o->precond == SG_PRECOND_DIAG) ? build_diag(c) : build_bj3(c);
    if (rc == SG_OK) rc = prepare_operator(c);
    if (rc == SG_OK && o->precond == SG_PRECOND_LEARNED && c->learned_kind == 1)
      rc = ensure_patches(c);
    if (rc) return rc;
    Job& j = jobs[i];
    j.c = c;
    j.pc = (o->precond == SG_PRECOND_BJ3) ? 1 : (o->precond == SG_PRECOND_DIAG ? 0 : 2);
    if (j.pc == 2 && !c->learned_enabled) {
      j.pc = 1;
      j.fallback = 0;
    }
    c->refresh_chi2 = false;  // no printed lines in a batch
    cudaEventCreateWithFlags(&j.ready, cudaEventDisableTiming);
    if (!c->ev0) cudaEventCreate(&c->ev0);
    if (!c->ev1) cudaEventCreate(&c->ev1);
    c->crit_hist.clear();
    j.launches0 = c->launches;
  }
  const int refresh_every = o->refresh_every > 0 ? o->refresh_every : 10;
  const int maxiter = o->maxiter > 0 ? o->maxiter : 2000;
  const char* dl_env = getenv("SANEPIC_GPU_DEVICE_LOOP");
  if (o->use_graph && !(dl_env && dl_env[0] == '0')) {
    const int rc = solve_batch_device(jobs, o, maxiter, refresh_every, reports);
    for (auto& j : jobs)
      if (j.ready) cudaEventDestroy(j.ready);
    return rc;
  }
  const double t0 = now_s();
  cudaError_t e = cudaSuccess;
  int failed = -1;
  for (int i = 0; i < n && e == cudaSuccess; i++) {
    sg_ctx* c = jobs[i].c;
    cudaSetDevice(c->desc.device);
    e = cudaEventRecord(c->ev0, c->st);
    if (e == cudaSuccess) e = enqueue_start(c, jobs[i].pc);
    if (e == cudaSuccess) e = enqueue_scalars(jobs[i]);
    if (e != cudaSuccess) failed = i;
  }
  int active = n;
  while (active > 0 && e == cudaSuccess) {
    bool progressed = false;
    for (int i = 0; i < n && e == cudaSuccess; i++) {
      Job& j = jobs[i];
      if (j.done || !j.pending) continue;
      const cudaError_t q = cudaEventQuery(j.ready);
      if (q == cudaErrorNotReady) continue;
      if (q != cudaSuccess) {
        e = q;
        failed = i;
        break;
      }
      progressed = true;
      j.pending = false;
      sg_ctx* c = j.c;
      cudaSetDevice(c->desc.device);
      if (!j.started) {
        j.started = true;
        j.var00 = c->sc_host->var00;
        j.crit = c->sc_host->var / j.var00;
      } else {
        j.crit = c->sc_host->var / j.var00;
        c->crit_hist.push_back(j.crit);
        j.iter++;
        const bool stop = j.crit <= o->stop_crit || j.iter >= maxiter;
        if (!stop && c->sc_host->flag && j.pc == 2) {
          // the network broke flexible PCG: restart with block-Jacobi
          j.fallback = j.iter;
          j.pc = 1;
          CgVecs v1 = c->vecs(1);
          e = c->apply_dev(c->x.as<double>(), c->r.as<double>(), true);
          if (e == cudaSuccess) e = c->f32 ? cg_init<float>(v1, c->st) : cg_init<double>(v1, c->st);
          if (e == cudaSuccess) e = c->to_map(c->d.as<double>());
          c->launches += 7;
          if (e == cudaSuccess) e = enqueue_scalars(j);
          if (e != cudaSuccess) failed = i;
          continue;
        }
        if (stop || c->sc_host->flag) {
          j.done = true;
          j.t_done = now_s();
          e = cudaEventRecord(c->ev1, c->st);
          active--;
          continue;
        }
      }
      e = c->run_iteration(j.pc, refresh_at(j.iter, refresh_every, j.pc != 0 ? 1 : 0),
                           o->use_graph != 0);
      if (e == cudaSuccess) e = enqueue_scalars(j);
      if (e != cudaSuccess) failed = i;
    }
    if (!progressed) std::this_thread::yield();
  }
  for (int i = 0; i < n; i++) {
    Job& j = jobs[i];
    sg_ctx* c = j.c;
    cudaSetDevice(c->desc.device);
    float ms = 0.f;
    if (e == cudaSuccess && j.done) {
      cudaEventSynchronize(c->ev1);
      cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    }
    if (j.ready) cudaEventDestroy(j.ready);
    c->have_solution = e == cudaSuccess;
    if (reports) {
      sg_report& r = reports[i];
      r = sg_report{};
      r.iterations = j.iter;
      r.converged = j.crit <= o->stop_crit;
      r.crit = j.crit;
      r.var00 = j.var00;
      r.solve_seconds = j.t_done - t0;
      r.iter_per_sec = j.iter / (j.t_done - t0 > 0 ? j.t_done - t0 : 1e-30);
      r.device_seconds = ms * 1e-3;
      r.kernel_launches = (long)(c->launches - j.launches0);
      r.breakdown = c->sc_host->flag;
      r.fallback_iter = j.fallback;
    }
  }
  if (e != cudaSuccess) {
    sg_ctx* c = jobs[failed >= 0 ? failed : 0].c;
    return c->cuda_fail(e, "batch solve");
  }
  return SG_OK;
}
