// Context lifetime, the field registry and the C ABI entry points that act on
// a context (include/xcore_gb300.h).
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <vector>
#include <unordered_map>
#include <mutex>

#include "xc_internal.cuh"

namespace {

thread_local char g_err[512] = "";

struct FieldInfo { const char* name; int shape; int elem; };
const FieldInfo kFields[FLD_COUNT] = {
#define XC_INFO(name, sh, eb) {#name, sh, eb},
    XC_FIELDS(XC_INFO)
#undef XC_INFO
};

size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

bool bc_ok(int b) { return b == XC_PERIODIC || b == XC_CLOSED; }

__global__ void seed_phase_kernel(int n, const double* rho, const double* x, const double* m,
                                  double* X, double* M) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  X[t] = rho[t] * x[t];
  M[t] = rho[t] * m[t];
}

int check_ctx(const xc_ctx* c) {
  if (!c) { xc_set_error("null context"); return XC_BAD_ARG; }
  return XC_OK;
}

}  // namespace

void xc_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

extern "C" const char* xc_last_error(void) { return g_err; }

unsigned persistent_grid(const void* kernel, int rows, int cols) {
  static std::mutex mu;
  static std::unordered_map<const void*, int> per_sm;   // resident CTAs of 256 threads per SM
  static int sms = 0;
  int b = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (sms == 0) {
      int dev = 0;
      cudaGetDevice(&dev);
      if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    }
    auto it = per_sm.find(kernel);
    if (it == per_sm.end()) {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, 256, 0) != cudaSuccess || b < 1) b = 1;
      cudaGetLastError();
      per_sm[kernel] = b;
    } else {
      b = it->second;
    }
  }
  const long long tiles = (long long)((rows + 31) / 32) * ((cols + 7) / 8);
  const long long wave = (long long)sms * b;
  return (unsigned)(tiles < wave ? tiles : wave);
}
extern "C" const char* xc_version(void) { return "xcore_gb300 0.1 (sm_103a)"; }

extern "C" int xc_field_count(void) { return FLD_COUNT; }
extern "C" const char* xc_field_name(int id) {
  return (id >= 0 && id < FLD_COUNT) ? kFields[id].name : nullptr;
}
extern "C" int xc_field_id(const char* name) {
  if (!name) return -1;
  for (int k = 0; k < FLD_COUNT; ++k)
    if (std::strcmp(kFields[k].name, name) == 0) return k;
  return -1;
}

extern "C" int xc_time_coefs(int tint, int step, double out[6]) {
  // src/timing.jl:18-36
  const double be[6] = {1, 1, 0, 1, 0, 0};
  const double bd2[6] = {1.5, 2.0, -0.5, 1, 0, 0};
  const double cn[6] = {1, 1, 0, 0.5, 0.5, 0};
  const double bd2si[6] = {1.5, 2.0, -0.5, 0.75, 0.5, -0.25};
  const double* r = nullptr;
  switch (tint) {
    case XC_BE1IM: r = be; break;
    case XC_BD2IM: r = step <= 2 ? be : bd2; break;
    case XC_CN2SI: r = step == 1 ? be : cn; break;
    case XC_BD2SI: r = step == 1 ? be : (step == 2 ? cn : bd2si); break;
    default:
      xc_set_error("time_coefs: unsupported TINT scheme %d", tint);
      return XC_BAD_ARG;
  }
  std::memcpy(out, r, sizeof(double) * 6);
  return XC_OK;
}

extern "C" int xc_ctx_create(const xc_params* par, xc_ctx** out) {
  if (!par || !out) { xc_set_error("xc_ctx_create: null argument"); return XC_BAD_ARG; }
  *out = nullptr;
  if (par->Nz < 3 || par->Nx < 3 || !(par->h > 0) || !bc_ok(par->xBC) || !bc_ok(par->zBC) ||
      par->ADVN < XC_CENTR || par->ADVN > XC_TVDIM || par->TINT < 0 || par->TINT > 3 ||
      par->weno_weights < 0 || par->weno_weights > 1) {
    xc_set_error("xc_ctx_create: bad parameters (Nz=%d Nx=%d h=%g ADVN=%d TINT=%d weno_weights=%d)", par->Nz,
                 par->Nx, par->h, par->ADVN, par->TINT, par->weno_weights);
    return XC_BAD_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    xc_set_error("xc_ctx_create: no CUDA device");
    return XC_NO_DEVICE;
  }
  xc_ctx* c = new xc_ctx();
  std::memset((void*)c, 0, sizeof(xc_ctx));
  c->p = *par;
  c->Nz = par->Nz;
  c->Nx = par->Nx;
  cudaGetDevice(&c->device);
  auto fail = [&](int st) { xc_ctx_destroy(c); return st; };
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess) {
    xc_set_error("xc_ctx_create: stream creation failed");
    return fail(XC_CUDA);
  }
  size_t total = 0;
  std::vector<size_t> off(FLD_COUNT);
  for (int k = 0; k < FLD_COUNT; ++k) {
    c->shape[k] = shape_of(kFields[k].shape, c->Nz, c->Nx);
    c->elem[k] = kFields[k].elem;
    off[k] = total;
    total += align256((size_t)c->shape[k].rows * c->shape[k].cols * c->elem[k]);
  }
  const size_t tmpn = align256(sizeof(double) * (size_t)(c->Nz + 2) * (c->Nx + 2) + 4096);
  const size_t tmp_off = total;
  total += 8 * tmpn;
  if (cudaMalloc(&c->arena, total) != cudaSuccess) {
    xc_set_error("xc_ctx_create: cannot allocate %zu bytes of device memory", total);
    return fail(XC_CUDA);
  }
  c->arena_bytes = total;
  if (cudaMemsetAsync(c->arena, 0, total, c->stream) != cudaSuccess) return fail(XC_CUDA);
  for (int k = 0; k < FLD_COUNT; ++k) c->field[k] = c->own[k] = c->arena + off[k];
  for (int k = 0; k < 8; ++k) c->tmp[k] = (double*)(c->arena + tmp_off + k * tmpn);
  c->red_partials_len = reduce_partials_len();
  if (cudaMalloc(&c->red_partials, sizeof(double) * c->red_partials_len) != cudaSuccess ||
      cudaMalloc(&c->red_partials_side, sizeof(double) * c->red_partials_len) != cudaSuccess ||
      cudaMalloc(&c->dscal, sizeof(double) * 64) != cudaSuccess ||
      cudaMallocHost(&c->hscal, sizeof(double) * 64) != cudaSuccess) {
    xc_set_error("xc_ctx_create: scratch allocation failed");
    return fail(XC_CUDA);
  }
  cudaMemsetAsync(c->dscal, 0, sizeof(double) * 64, c->stream);
  // the arrival counters at the end of each reduction scratch start at zero
  cudaMemsetAsync(c->red_partials, 0, sizeof(double) * c->red_partials_len, c->stream);
  cudaMemsetAsync(c->red_partials_side, 0, sizeof(double) * c->red_partials_len, c->stream);
  int st = noise_plan_create(c);
  if (st != XC_OK) return fail(st);
  st = stokes_create(c);
  if (st != XC_OK) return fail(st);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
    xc_set_error("xc_ctx_create: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(XC_CUDA);
  }
  *out = c;
  return XC_OK;
}

extern "C" int xc_ctx_destroy(xc_ctx* c) {
  if (!c) return XC_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->side) cudaStreamSynchronize(c->side);
  noise_plan_destroy(c);
  stokes_destroy(c);
  if (c->arena) cudaFree(c->arena);
  if (c->red_partials) cudaFree(c->red_partials);
  if (c->red_partials_side) cudaFree(c->red_partials_side);
  if (c->dscal) cudaFree(c->dscal);
  if (c->hscal) cudaFreeHost(c->hscal);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  delete c;
  return XC_OK;
}

extern "C" int xc_field_shape(const xc_ctx* c, int id, int* rows, int* cols, int* elem_bytes) {
  XC_TRY(check_ctx(c));
  if (id < 0 || id >= FLD_COUNT) { xc_set_error("bad field id %d", id); return XC_BAD_ARG; }
  if (rows) *rows = c->shape[id].rows;
  if (cols) *cols = c->shape[id].cols;
  if (elem_bytes) *elem_bytes = c->elem[id];
  return XC_OK;
}

extern "C" int xc_field_device_ptr(const xc_ctx* c, int id, void** dev_ptr) {
  XC_TRY(check_ctx(c));
  if (id < 0 || id >= FLD_COUNT || !dev_ptr) { xc_set_error("bad field id %d", id); return XC_BAD_ARG; }
  *dev_ptr = c->field[id];
  return XC_OK;
}

extern "C" int xc_field_bind(xc_ctx* c, int id, void* dev_ptr) {
  XC_TRY(check_ctx(c));
  if (id < 0 || id >= FLD_COUNT) { xc_set_error("xc_field_bind: bad field id %d", id); return XC_BAD_ARG; }
  if (((uintptr_t)dev_ptr & 15u) != 0) {
    xc_set_error("xc_field_bind: field %s: device pointer not 16-byte aligned", kFields[id].name);
    return XC_BAD_ARG;
  }
  if (dev_ptr) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, dev_ptr) != cudaSuccess ||
        (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
      cudaGetLastError();
      xc_set_error("xc_field_bind: field %s: not a device pointer", kFields[id].name);
      return XC_BAD_ARG;
    }
  }
  XC_CUDA_TRY(cudaStreamSynchronize(c->stream));
  XC_CUDA_TRY(cudaStreamSynchronize(c->side));
  c->field[id] = dev_ptr ? dev_ptr : c->own[id];
  return XC_OK;
}

extern "C" int xc_field_upload(xc_ctx* c, int id, const void* host) {
  XC_TRY(check_ctx(c));
  if (id < 0 || id >= FLD_COUNT || !host) { xc_set_error("bad field id %d", id); return XC_BAD_ARG; }
  size_t n = (size_t)c->shape[id].rows * c->shape[id].cols * c->elem[id];
  XC_CUDA_TRY(cudaMemcpyAsync(c->field[id], host, n, cudaMemcpyHostToDevice, c->stream));
  XC_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return XC_OK;
}

extern "C" int xc_field_download(xc_ctx* c, int id, void* host) {
  XC_TRY(check_ctx(c));
  if (id < 0 || id >= FLD_COUNT || !host) { xc_set_error("bad field id %d", id); return XC_BAD_ARG; }
  size_t n = (size_t)c->shape[id].rows * c->shape[id].cols * c->elem[id];
  XC_CUDA_TRY(cudaMemcpyAsync(host, c->field[id], n, cudaMemcpyDeviceToHost, c->stream));
  XC_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return XC_OK;
}

extern "C" int xc_synchronize(xc_ctx* c) {
  XC_TRY(check_ctx(c));
  XC_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return XC_OK;
}

extern "C" int xc_store_previous(xc_ctx* c) { XC_TRY(check_ctx(c)); return store_previous_impl(c); }
extern "C" int xc_store_noise(xc_ctx* c) { XC_TRY(check_ctx(c)); return store_noise_impl(c); }
extern "C" int xc_snapshot(xc_ctx* c) { XC_TRY(check_ctx(c)); return snapshot_impl(c); }

extern "C" int xc_phsevo(xc_ctx* c, int scheme, const double coefs[6], double dt, double alpha) {
  XC_TRY(check_ctx(c));
  if (!coefs) { xc_set_error("xc_phsevo: null coefs"); return XC_BAD_ARG; }
  if (scheme < 0) scheme = c->p.ADVN;
  if (scheme > XC_TVDIM) { xc_set_error("xc_phsevo: unknown scheme %d", scheme); return XC_BAD_ARG; }
  return phsevo_impl(c, scheme, coefs, dt, alpha);
}

extern "C" int xc_fluidmech(xc_ctx* c, const double coefs[6], double dt, const xc_solver_opts* opts,
                            xc_solver_stats* stats) {
  XC_TRY(check_ctx(c));
  if (!coefs) { xc_set_error("xc_fluidmech: null coefs"); return XC_BAD_ARG; }
  return fluidmech_impl(c, coefs, dt, opts, stats, nullptr);
}

extern "C" int xc_fluidmech_mms(xc_ctx* c, const double* src_W, const double* src_U,
                                const double* src_P, const double* W_exact, const double* U_exact,
                                const double* P_exact, const double coefs[6], double dt,
                                const xc_solver_opts* opts, xc_solver_stats* stats) {
  XC_TRY(check_ctx(c));
  if (!coefs || !src_W || !src_U || !src_P || !W_exact || !U_exact || !P_exact) {
    xc_set_error("xc_fluidmech_mms: null argument");
    return XC_BAD_ARG;
  }
  MmsData m{src_W, src_U, src_P, W_exact, U_exact, P_exact};
  return fluidmech_impl(c, coefs, dt, opts, stats, &m);
}

extern "C" int xc_noise(xc_ctx* c, double dt, int first_iter, const double* re, const double* rs) {
  XC_TRY(check_ctx(c));
  return noise_impl(c, dt, first_iter, re, rs);
}

extern "C" int xc_update_phase_velocities(xc_ctx* c) {
  XC_TRY(check_ctx(c));
  return phase_velocities_impl(c);
}

extern "C" int xc_update(xc_ctx* c) { XC_TRY(check_ctx(c)); return update_impl(c); }

extern "C" int xc_update_dt(xc_ctx* c, double dt_prev, double* dt_out) {
  XC_TRY(check_ctx(c));
  if (!dt_out) { xc_set_error("xc_update_dt: null output"); return XC_BAD_ARG; }
  return update_dt_impl(c, dt_prev, dt_out);
}

extern "C" int xc_resnorm(xc_ctx* c, double dt, double out[3]) {
  XC_TRY(check_ctx(c));
  if (!out) { xc_set_error("xc_resnorm: null output"); return XC_BAD_ARG; }
  return resnorm_impl(c, dt, out);
}

extern "C" int xc_conservation_sums(xc_ctx* c, double out[12]) {
  XC_TRY(check_ctx(c));
  if (!out) { xc_set_error("xc_conservation_sums: null output"); return XC_BAD_ARG; }
  return sums_impl(c, out);
}

extern "C" int xc_history_stats(xc_ctx* c, double out[58]) {
  XC_TRY(check_ctx(c));
  if (!out) { xc_set_error("xc_history_stats: null output"); return XC_BAD_ARG; }
  return history_impl(c, out);
}

static int upload_async(xc_ctx* c, int id, const void* host) {
  size_t n = (size_t)c->shape[id].rows * c->shape[id].cols * c->elem[id];
  XC_CUDA_TRY(cudaMemcpyAsync(c->field[id], host, n, cudaMemcpyHostToDevice, c->stream));
  return XC_OK;
}

static int dcopy(xc_ctx* c, int dst, int src) {
  size_t n = (size_t)c->shape[src].rows * c->shape[src].cols * c->elem[src];
  XC_CUDA_TRY(cudaMemcpyAsync(c->field[dst], c->field[src], n, cudaMemcpyDeviceToDevice, c->stream));
  return XC_OK;
}

// initialize! fresh-start branch (src/run.jl:89-130)
extern "C" int xc_initialize(xc_ctx* c, const double* x_init, const double* re, const double* rs) {
  XC_TRY(check_ctx(c));
  if (!x_init || !re || !rs) { xc_set_error("xc_initialize: null argument"); return XC_BAD_ARG; }
  const int Nz = c->Nz, Nx = c->Nx;
  const xc_params& p = c->p;
  // compute_bndtaperw! / compute_bndshape! (run.jl:24-55), host scalars
  std::vector<double> taper((size_t)(Nz + 1) * (Nx + 2)), shape((size_t)Nz * Nx);
  const double osgr = p.open_sgr ? 1.0 : 0.0;
  for (int i = 0; i < Nx + 2; ++i)
    for (int j = 0; j <= Nz; ++j) {
      double z = (double)j * p.h;
      taper[(size_t)i * (Nz + 1) + j] = 1.0 - (std::exp(-z / p.l0h) + std::exp(-(p.D - z) / p.l0h)) * (1.0 - osgr);
    }
  for (int i = 0; i < Nx; ++i)
    for (int j = 0; j < Nz; ++j) {
      double zc = ((double)(j + 1) - 0.5) * p.h;
      shape[(size_t)i * Nz + j] = std::exp((-zc + p.h / 2.0) / p.bnd_w);
    }
  std::vector<double> m((size_t)Nz * Nx), e0((size_t)(Nz + 1) * (Nx + 1), p.etam0);
  for (size_t k = 0; k < m.size(); ++k) m[k] = 1.0 - x_init[k];
  XC_TRY(upload_async(c, FLD_bndtaperw, taper.data()));
  XC_TRY(upload_async(c, FLD_bndshape, shape.data()));
  XC_TRY(upload_async(c, FLD_x, x_init));
  XC_TRY(upload_async(c, FLD_m, m.data()));
  XC_TRY(upload_async(c, FLD_eta, e0.data()));
  XC_TRY(upload_async(c, FLD_etaco, e0.data()));
  XC_TRY(upload_async(c, FLD_etas, e0.data()));
  XC_TRY(update_impl(c));
  const int n = Nz * Nx;
  seed_phase_kernel<<<(n + 255) / 256, 256, 0, c->stream>>>(
      n, (const double*)c->field[FLD_rho], (const double*)c->field[FLD_x],
      (const double*)c->field[FLD_m], (double*)c->field[FLD_X], (double*)c->field[FLD_M]); xc_count_launch();
  XC_LAUNCH_CHECK();
  XC_TRY(noise_impl(c, p.dt0, 1, re, rs));
  XC_TRY(phase_velocities_impl(c));
  XC_TRY(dcopy(c, FLD_Xo, FLD_X));
  XC_TRY(dcopy(c, FLD_Xoo, FLD_X));
  XC_TRY(dcopy(c, FLD_Mo, FLD_M));
  XC_TRY(dcopy(c, FLD_Moo, FLD_M));
  XC_TRY(dcopy(c, FLD_rhoo, FLD_rho));
  XC_TRY(dcopy(c, FLD_rhooo, FLD_rho));
  XC_TRY(store_noise_impl(c));
  XC_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return XC_OK;
}

// One outer step of run! (src/run.jl:204-274).  fixed_sweeps > 0 runs exactly
// that many Picard sweeps; fixed_sweeps == 0 runs the reference's while-loop
// (run.jl:220-250) with rtol / atol / maxit.
static int step_impl(xc_ctx* c, int step, double dt, int fixed_sweeps, double rtol, double atol, int maxit,
                     const double* re, const double* rs, const xc_solver_opts* opts, xc_step_stats* stats) {
  double coefs[6];
  XC_TRY(xc_time_coefs(c->p.TINT, step, coefs));
  XC_TRY(store_previous_impl(c));
  XC_TRY(store_noise_impl(c));
  xc_step_stats local;
  std::memset(&local, 0, sizeof(local));
  // the main stream waits for the side stream's noise! before it goes on
  auto join = [&]() -> int {
    XC_CUDA_TRY(cudaEventRecord(c->ev_join, c->side));
    XC_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    return XC_OK;
  };
  auto finish = [&](int st) {
    if (stats) *stats = local;
    return st;
  };
  double resnorm = 1.0, resnorm0 = 1.0;
  int it = 0;
  auto more = [&]() {
    if (fixed_sweeps > 0) return it < fixed_sweeps;
    return (resnorm / resnorm0 >= rtol && resnorm >= atol && it < maxit) || it < 3;
  };
  while (more()) {
    ++it;
    local.sweeps = it;
    XC_TRY(finish(snapshot_impl(c)));
    int st = phsevo_impl(c, c->p.ADVN, coefs, dt, c->p.alpha);
    if (st != XC_OK) return finish(st);
    // noise! (run.jl:240) reads only what the previous update! (or the
    // initial state) left -- V, vx, fReL, ke, ks, chi, the face fractions and
    // the stored noise -- none of which phsevo! or fluidmech! write, and
    // neither of them reads its results: it runs on the side stream beside
    // the latency-bound iterations of the Stokes solve (forked once the
    // solve's FP64 right-hand side and setup are enqueued), and
    // update_phase_velocities! waits for it
    bool forked = false;
    int nst = XC_OK;
    const std::function<int()> fork_noise = [&]() -> int {
      forked = true;
      XC_CUDA_TRY(cudaEventRecord(c->ev_fork, c->stream));
      XC_CUDA_TRY(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
      nst = noise_impl(c, dt, it == 1, it == 1 ? re : nullptr, it == 1 ? rs : nullptr, c->side,
                       c->red_partials_side);
      return XC_OK;
    };
    xc_solver_stats ss;
    std::memset(&ss, 0, sizeof(ss));
    st = fluidmech_impl(c, coefs, dt, opts, &ss, nullptr, &fork_noise);
    if (!forked) fork_noise();   // a solve that returned before its iterations
    if (nst != XC_OK) { join(); return finish(nst); }
    XC_TRY(finish(join()));
    // a solve that stopped at its iteration cap leaves a usable iterate; the
    // step goes on as the reference's would and reports it at the end
    if (st == XC_NOT_CONVERGED) ++local.unconverged_solves;
    else if (st != XC_OK) return finish(st);
    local.solver_iterations += ss.iterations;
    if (ss.rel_residual > local.solver_rel_residual) local.solver_rel_residual = ss.rel_residual;
    XC_TRY(finish(phase_velocities_impl(c)));
    XC_TRY(finish(update_impl(c)));
    double rn[3];
    XC_TRY(finish(resnorm_impl(c, dt, rn)));
    resnorm = rn[0];
    local.resnorm[it - 1] = resnorm;
    // set the reference on the first sweep, raise it when the residual grew
    // (run.jl:246-249)
    if (it == 1 || resnorm > resnorm0) resnorm0 = resnorm + 1e-32;
    local.resnorm0 = resnorm0;
    if (std::isnan(resnorm)) {
      xc_set_error("Solver diverged with NaN at iter %d", it);
      return finish(XC_NAN);
    }
  }
  if (fixed_sweeps == 0) local.picard_converged = (resnorm / resnorm0 < rtol || resnorm < atol) ? 1 : 0;
  XC_TRY(finish(update_dt_impl(c, dt, &local.dt_next)));
  if (local.unconverged_solves > 0) {
    xc_set_error("step %d: %d of %d Stokes solves stopped at their iteration cap (worst relative residual "
                 "%.3e); the step was completed with those iterates", step, local.unconverged_solves, it,
                 local.solver_rel_residual);
    return finish(XC_NOT_CONVERGED);
  }
  return finish(XC_OK);
}

extern "C" int xc_step(xc_ctx* c, int step, double dt, int sweeps, const double* re,
                       const double* rs, const xc_solver_opts* opts, xc_step_stats* stats) {
  XC_TRY(check_ctx(c));
  if (sweeps < 1 || sweeps > XC_MAX_SWEEPS) {
    xc_set_error("xc_step: sweeps must be 1..%d", XC_MAX_SWEEPS);
    return XC_BAD_ARG;
  }
  return step_impl(c, step, dt, sweeps, 0.0, 0.0, sweeps, re, rs, opts, stats);
}

extern "C" int xc_step_converge(xc_ctx* c, int step, double dt, double rtol, double atol, int maxit,
                                const double* re, const double* rs, const xc_solver_opts* opts,
                                xc_step_stats* stats) {
  XC_TRY(check_ctx(c));
  if (maxit < 0 || maxit > XC_MAX_SWEEPS || !(rtol >= 0) || !(atol >= 0)) {
    xc_set_error("xc_step_converge: need 0 <= maxit <= %d and rtol, atol >= 0", XC_MAX_SWEEPS);
    return XC_BAD_ARG;
  }
  return step_impl(c, step, dt, 0, rtol, atol, maxit, re, rs, opts, stats);
}

extern "C" int xc_print_step_stats(xc_ctx* c, double out[24]) {
  XC_TRY(check_ctx(c));
  if (!out) { xc_set_error("xc_print_step_stats: null output"); return XC_BAD_ARG; }
  return print_stats_impl(c, out);
}

// ---------------------------------------------------------------------------
// instrumentation
// ---------------------------------------------------------------------------
std::atomic<long long> g_xc_launches{0};
thread_local long long g_xc_thread_launches = 0;

extern "C" void* xc_stream(xc_ctx* c) { return c ? (void*)c->stream : nullptr; }
extern "C" long long xc_launch_count(void) { return g_xc_launches.load(); }

int noise_bench_zpass(xc_ctx* c, int iters, double out[4]);

extern "C" int xc_bench_kernel(xc_ctx* c, int which, int iters, double out[4]) {
  XC_TRY(check_ctx(c));
  if (!out || iters < 1) { xc_set_error("xc_bench_kernel: bad arguments"); return XC_BAD_ARG; }
  if (which == 1 || which == 2 || which == 3 || which == 5) return stokes_bench(c, which, iters, out);
  if (which == 4) return noise_bench_zpass(c, iters, out);
  if (which != 0) { xc_set_error("xc_bench_kernel: unknown kernel %d", which); return XC_BAD_ARG; }
  const int Nz = c->Nz, Nx = c->Nx;
  DView Wx = F(c, FLD_Wx), Ux = F(c, FLD_Ux), X = F(c, FLD_X);
  CView Wx_face{Wx.p + Wx.ld, Wx.ld}, Ux_face{Ux.p + 1, Ux.ld};
  DView qx = F(c, FLD_qx_advn_X), qz = F(c, FLD_qz_advn_X);
  DView qxi{qx.p + 1, qx.ld}, qzi{qz.p + qz.ld, qz.ld};
  cudaEvent_t e0, e1;
  XC_CUDA_TRY(cudaEventCreate(&e0));
  XC_CUDA_TRY(cudaEventCreate(&e1));
  int st = XC_OK;
  for (int it = -1; it < iters && st == XC_OK; ++it) {
    if (it == 0) cudaEventRecord(e0, c->stream);
    st = stencil_advect_flux(X.p, X.ld, false, Nz, Nx, advect_scheme(c->p.ADVN, c->p), c->p.xBC, c->p.zBC, Ux_face, Wx_face, c->p.h,
                             F(c, FLD_advn_X), qxi, qzi, c->stream);
  }
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != XC_OK) return st;
  const double cells = (double)Nz * Nx;
  // WENO5: two upwind reconstructions per cell (one x face, one z face) of
  // about 66 flops with 4 divisions each (1 with weno_weights = 1), the flux
  // products and the divergence
  const double fpc = c->p.ADVN == XC_WENO5 ? 150.0 : (c->p.ADVN == XC_QUICK ? 38.0 : 20.0);
  out[0] = ms / iters;
  out[1] = 48.0 * cells;     // read f, u, w; write adv, qx, qz (8 B each per cell)
  out[2] = fpc * cells;
  out[3] = cells;
  return XC_OK;
}
