// Ensembles of independent contexts (uneven grid sizes, parameters and noise
// seeds) advanced by one time step together.  Every explicit stage of a
// Picard sweep is one CUDA graph launch for the whole ensemble: the stage's
// kernels of all members, captured once from the members' own streams into
// one graph whose member branches run side by side on the GPU --
//
//   pre   store_previous! + store_noise! (first sweep), snapshot!, phsevo!
//   noise noise! (beside the Stokes solves, as xc_step runs it)
//   post  update_phase_velocities!, update!, compute_resnorm's reductions
//   dt    update_dt's reductions (after the last sweep)
//
// -- and the members' Stokes solves (fluidmech!, host-driven FGMRES) run
// concurrently on a pool of host threads, one member per thread at a time, each
// on its member's stream.  The kernels, their arguments and their order per
// member are those of xc_step with a fixed number of sweeps, so every member
// ends bit-identical to the same context stepped alone.  The pre and noise
// graphs hold the step's dt and time coefficients and are re-captured each step
// (and updated in place when their topology is unchanged); post and dt are
// captured once.
#include <cmath>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "xc_internal.cuh"
#include "xc_pool.h"

namespace {

struct Stage {
  cudaGraphExec_t exec = nullptr;
  long long kernels = 0;   // kernel nodes of the graph (library launches it stands for)
};

}  // namespace

struct xc_ensemble {
  std::vector<xc_ctx*> m;
  int device = 0;
  cudaStream_t es = nullptr, es2 = nullptr;   // where the stage graphs run
  cudaEvent_t ev_fork = nullptr, ev_pre = nullptr, ev_noise = nullptr;
  std::vector<cudaEvent_t> ev_m;              // per member: joins its branch back
  Stage pre_first, pre_rest, noise, post, dt;
  xc::WorkerPool* pool = nullptr;
};

namespace {

void destroy_stage(Stage& st) {
  if (st.exec) cudaGraphExecDestroy(st.exec);
  st.exec = nullptr;
}

// Capture body(i) of every member into one graph: each member's stream (its
// side stream when `side`) joins the capture from e->es, body enqueues that
// member's stage on it, and the branch is joined back before the capture
// ends.  The executable graph is updated in place when one exists and the
// topology allows, instantiated otherwise.
int capture_stage(xc_ensemble* e, Stage& st, bool side, const std::function<int(int)>& body) {
  const long long before = g_xc_thread_launches;
  XC_CUDA_TRY(cudaStreamBeginCapture(e->es, cudaStreamCaptureModeThreadLocal));
  int status = XC_OK;
  cudaError_t ce = cudaEventRecord(e->ev_fork, e->es);
  for (size_t i = 0; i < e->m.size() && ce == cudaSuccess && status == XC_OK; ++i) {
    xc_ctx* c = e->m[i];
    cudaStream_t s = side ? c->side : c->stream;
    ce = cudaStreamWaitEvent(s, e->ev_fork, 0);
    if (ce != cudaSuccess) break;
    status = body((int)i);
    if (status != XC_OK) break;
    ce = cudaEventRecord(e->ev_m[i], s);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(e->es, e->ev_m[i], 0);
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(e->es, &graph);
  const long long kernels = g_xc_thread_launches - before;
  g_xc_thread_launches = before;             // captured, not launched
  g_xc_launches.fetch_sub(kernels);
  if (status != XC_OK || ce != cudaSuccess || ee != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    if (status != XC_OK) return status;
    xc_set_error("ensemble: stage capture failed: %s",
                 cudaGetErrorString(ce != cudaSuccess ? ce : ee));
    return XC_CUDA;
  }
  if (st.exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(st.exec, graph, &info) != cudaSuccess) {
      cudaGetLastError();
      destroy_stage(st);
    }
  }
  cudaError_t ie = cudaSuccess;
  if (!st.exec) ie = cudaGraphInstantiate(&st.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    st.exec = nullptr;
    xc_set_error("ensemble: graph instantiation failed: %s", cudaGetErrorString(ie));
    return XC_CUDA;
  }
  st.kernels = kernels;
  return XC_OK;
}

int launch_stage(const Stage& st, cudaStream_t s) {
  XC_CUDA_TRY(cudaGraphLaunch(st.exec, s));
  g_xc_launches.fetch_add(st.kernels);
  g_xc_thread_launches += st.kernels;
  return XC_OK;
}

// every member's device scalars [first, first + n) to its pinned host mirror,
// then wait for e->es
int fetch_all(xc_ensemble* e, int first, int n) {
  for (xc_ctx* c : e->m)
    XC_CUDA_TRY(cudaMemcpyAsync(c->hscal + first, c->dscal + first, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                e->es));
  XC_CUDA_TRY(cudaStreamSynchronize(e->es));
  return XC_OK;
}

}  // namespace

extern "C" int xc_ensemble_destroy(xc_ensemble* e) {
  if (!e) return XC_OK;
  if (e->es) cudaStreamSynchronize(e->es);
  if (e->es2) cudaStreamSynchronize(e->es2);
  delete e->pool;
  for (Stage* st : {&e->pre_first, &e->pre_rest, &e->noise, &e->post, &e->dt}) destroy_stage(*st);
  for (cudaEvent_t ev : e->ev_m)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : {e->ev_fork, e->ev_pre, e->ev_noise})
    if (ev) cudaEventDestroy(ev);
  if (e->es) cudaStreamDestroy(e->es);
  if (e->es2) cudaStreamDestroy(e->es2);
  delete e;
  return XC_OK;
}

extern "C" int xc_ensemble_create(xc_ctx* const* members, int n, int threads, xc_ensemble** out) {
  if (!out || !members || n < 1 || threads < 0) {
    xc_set_error("xc_ensemble_create: need members, n >= 1, threads >= 0 and out");
    return XC_BAD_ARG;
  }
  *out = nullptr;
  xc_ensemble* e = new xc_ensemble();
  e->m.assign(members, members + n);
  auto fail = [&](int st) {
    xc_ensemble_destroy(e);
    return st;
  };
  for (int i = 0; i < n; ++i) {
    if (!e->m[i]) {
      xc_set_error("xc_ensemble_create: member %d is null", i);
      return fail(XC_BAD_ARG);
    }
    for (int k = 0; k < i; ++k)
      if (e->m[k] == e->m[i]) {
        xc_set_error("xc_ensemble_create: members %d and %d are the same context", k, i);
        return fail(XC_BAD_ARG);
      }
    if (e->m[i]->device != e->m[0]->device) {
      xc_set_error("xc_ensemble_create: members on different devices (%d, %d)", e->m[0]->device,
                   e->m[i]->device);
      return fail(XC_BAD_ARG);
    }
  }
  e->device = e->m[0]->device;
  if (cudaSetDevice(e->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&e->es, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&e->es2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_pre, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_noise, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    xc_set_error("xc_ensemble_create: stream or event creation failed");
    return fail(XC_CUDA);
  }
  e->ev_m.assign(n, nullptr);
  for (int i = 0; i < n; ++i)
    if (cudaEventCreateWithFlags(&e->ev_m[i], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      xc_set_error("xc_ensemble_create: event creation failed");
      return fail(XC_CUDA);
    }
  e->pool = new xc::WorkerPool(threads > 0 ? (threads < n ? threads : n) : n, e->device);
  *out = e;
  return XC_OK;
}

extern "C" int xc_ensemble_step(xc_ensemble* e, const int* steps, const double* dts, int sweeps,
                                const double* const* re, const double* const* rs, const xc_solver_opts* opts,
                                xc_step_stats* stats) {
  if (!e || !steps || !dts) {
    xc_set_error("xc_ensemble_step: null argument");
    return XC_BAD_ARG;
  }
  if (sweeps < 1 || sweeps > XC_MAX_SWEEPS) {
    xc_set_error("xc_ensemble_step: sweeps must be 1..%d", XC_MAX_SWEEPS);
    return XC_BAD_ARG;
  }
  const int n = (int)e->m.size();
  XC_CUDA_TRY(cudaSetDevice(e->device));
  std::vector<double> coefs(6 * (size_t)n);
  for (int i = 0; i < n; ++i) XC_TRY(xc_time_coefs(e->m[i]->p.TINT, steps[i], &coefs[6 * (size_t)i]));
  std::vector<xc_step_stats> local(n);
  std::memset(local.data(), 0, sizeof(xc_step_stats) * n);
  // every return after the first enqueue: nothing of the step left running
  auto finish = [&](int st) {
    cudaStreamSynchronize(e->es2);
    cudaStreamSynchronize(e->es);
    if (stats) std::memcpy(stats, local.data(), sizeof(xc_step_stats) * n);
    return st;
  };
  // after the first enqueue every error return goes through finish()
#define ETRY(expr)                   \
  do {                               \
    const int st_ = (expr);          \
    if (st_ != XC_OK) return finish(st_); \
  } while (0)
#define ETRY_CUDA(call)                                                              \
  do {                                                                               \
    const cudaError_t ce_ = (call);                                                  \
    if (ce_ != cudaSuccess) {                                                        \
      xc_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(ce_)); \
      return finish(XC_CUDA);                                                        \
    }                                                                                \
  } while (0)
  // the graphs run on e->es: after everything already on the members' streams
  for (int i = 0; i < n; ++i) {
    xc_ctx* c = e->m[i];
    ETRY_CUDA(cudaEventRecord(e->ev_m[i], c->stream));
    ETRY_CUDA(cudaStreamWaitEvent(e->es, e->ev_m[i], 0));
    ETRY_CUDA(cudaEventRecord(e->ev_m[i], c->side));
    ETRY_CUDA(cudaStreamWaitEvent(e->es, e->ev_m[i], 0));
  }
  // the step's white-noise draws (xc_step copies them at the first sweep's noise!)
  for (int i = 0; i < n; ++i) {
    xc_ctx* c = e->m[i];
    const size_t nb = sizeof(double) * (size_t)c->Nz * c->Nx;
    if (re && re[i]) ETRY_CUDA(cudaMemcpyAsync(c->field[FLD_re], re[i], nb, cudaMemcpyHostToDevice, e->es));
    if (rs && rs[i]) ETRY_CUDA(cudaMemcpyAsync(c->field[FLD_rs], rs[i], nb, cudaMemcpyHostToDevice, e->es));
  }
  // this step's pre and noise stages (their kernels take dt and the time
  // coefficients); post and dt hold no per-step values
  ETRY(capture_stage(e, e->pre_first, false, [&](int i) {
    xc_ctx* c = e->m[i];
    XC_TRY(store_previous_impl(c));
    XC_TRY(store_noise_impl(c));
    XC_TRY(snapshot_impl(c));
    return phsevo_impl(c, c->p.ADVN, &coefs[6 * (size_t)i], dts[i], c->p.alpha);
  }));
  if (sweeps > 1)
    ETRY(capture_stage(e, e->pre_rest, false, [&](int i) {
      xc_ctx* c = e->m[i];
      XC_TRY(snapshot_impl(c));
      return phsevo_impl(c, c->p.ADVN, &coefs[6 * (size_t)i], dts[i], c->p.alpha);
    }));
  ETRY(capture_stage(e, e->noise, true, [&](int i) {
    xc_ctx* c = e->m[i];
    return noise_impl(c, dts[i], 1, nullptr, nullptr, c->side, c->red_partials_side);
  }));
  if (!e->post.exec)
    ETRY(capture_stage(e, e->post, false, [&](int i) {
      xc_ctx* c = e->m[i];
      XC_TRY(phase_velocities_impl(c));
      XC_TRY(update_impl(c));
      return resnorm_reduce(c);
    }));
  if (!e->dt.exec) ETRY(capture_stage(e, e->dt, false, [&](int i) { return update_dt_reduce(e->m[i]); }));

  std::vector<double> resnorm0(n, 1.0);
  std::vector<int> sst(n);
  std::vector<xc_solver_stats> ss(n);
  std::vector<std::string> serr(n);
  for (int it = 1; it <= sweeps; ++it) {
    ETRY(launch_stage(it == 1 ? e->pre_first : e->pre_rest, e->es));
    ETRY_CUDA(cudaEventRecord(e->ev_pre, e->es));
    // noise! reads only what the previous update! (or store_noise!) left,
    // which neither phsevo! nor fluidmech! writes: beside the solves
    ETRY_CUDA(cudaStreamWaitEvent(e->es2, e->ev_pre, 0));
    ETRY(launch_stage(e->noise, e->es2));
    ETRY_CUDA(cudaEventRecord(e->ev_noise, e->es2));
    // the Stokes solves, one member per pool thread; each returns once its
    // solve has finished on the device
    e->pool->run(n, [&](int i) {
      xc_ctx* c = e->m[i];
      std::memset(&ss[i], 0, sizeof(ss[i]));
      cudaError_t ce = cudaStreamWaitEvent(c->stream, e->ev_pre, 0);
      sst[i] = ce == cudaSuccess ? fluidmech_impl(c, &coefs[6 * (size_t)i], dts[i], opts, &ss[i], nullptr)
                                 : XC_CUDA;
      if (sst[i] != XC_OK) serr[i] = ce == cudaSuccess ? xc_last_error() : cudaGetErrorString(ce);
    });
    ETRY_CUDA(cudaStreamWaitEvent(e->es, e->ev_noise, 0));
    for (int i = 0; i < n; ++i) {
      local[i].sweeps = it;
      if (sst[i] == XC_NOT_CONVERGED) {
        ++local[i].unconverged_solves;
      } else if (sst[i] != XC_OK) {
        xc_set_error("ensemble member %d, sweep %d: %s", i, it, serr[i].c_str());
        return finish(sst[i]);
      }
      local[i].solver_iterations += ss[i].iterations;
      if (ss[i].rel_residual > local[i].solver_rel_residual) local[i].solver_rel_residual = ss[i].rel_residual;
    }
    ETRY(launch_stage(e->post, e->es));
    ETRY(fetch_all(e, SC_RESNORM, 9));
    int nan_member = -1;
    for (int i = 0; i < n; ++i) {
      double rn[3];
      resnorm_finish(e->m[i], dts[i], rn);
      local[i].resnorm[it - 1] = rn[0];
      if (it == 1 || rn[0] > resnorm0[i]) resnorm0[i] = rn[0] + 1e-32;
      local[i].resnorm0 = resnorm0[i];
      if (std::isnan(rn[0]) && nan_member < 0) nan_member = i;
    }
    if (nan_member >= 0) {
      xc_set_error("ensemble member %d: solver diverged with NaN at iter %d", nan_member, it);
      return finish(XC_NAN);
    }
  }
  ETRY(launch_stage(e->dt, e->es));
  ETRY(fetch_all(e, SC_DT, 5));
  int unconverged = 0;
  for (int i = 0; i < n; ++i) {
    update_dt_finish(e->m[i], dts[i], &local[i].dt_next);
    unconverged += local[i].unconverged_solves > 0;
  }
  if (unconverged > 0) {
    xc_set_error("ensemble step: %d of %d members had Stokes solves stopped at their iteration cap; their steps "
                 "were completed with those iterates", unconverged, n);
    return finish(XC_NOT_CONVERGED);
  }
  return finish(XC_OK);
#undef ETRY
#undef ETRY_CUDA
}
