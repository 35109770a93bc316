// Host side of the tangent-linear model and the discrete adjoint of N FP64
// do_step calls (splash_adjoint_* and splash_tlm_run of splash_gb300.h).
//
// An adjoint object borrows the geometry of an FP64 solver and owns its own
// state, checkpoints and tape:
//   forward   the FP64 step kernels from U0 with parameters theta; the
//             state every K steps is kept (checkpoints) and the dt of every
//             step is recorded (the schedule the derivatives freeze);
//   backward  per K-step interval, last first: recompute the interval from
//             its checkpoint storing each step's primal tape, then run the
//             reverse steps back to the interval start;
//   tlm       the same N steps on Dual<1> (value + one direction).
// theta = (accretion_rate, tilt_angle, omega_acc_abs) enters through the
// per-face accretion profile (physics/adiabatic.hpp:70-90, 415-421), the
// accretion angular velocity (0, sin tilt, cos tilt) omega_acc_abs and the
// depletion rate; the initial total mass (a function of U0) enters the
// depletion term when friction is off.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <vector>

#include "adjoint.hpp"
#include "kernels.hpp"
#include "layout.hpp"
#include "slot_planes.hpp"
#include "solver.hpp"
#include "splash_gb300.h"

namespace splash {
namespace {

#define ADJ_CUDA(call)                                                                            \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return set_error(SPLASH_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),    \
                       __FILE__, __LINE__);                                                       \
  } while (0)

}  // namespace

struct Adjoint {
  Solver* base = nullptr;
  int K = 50;
  int n_faces = 0, fpad = 0, max_slots = 0;
  size_t PS = 0, FS = 0;  // one slot-plane set / one face-plane set of 5 fields
  DevGeom G{};
  PhysParams P{};
  splash_params par{};
  std::vector<double> fcn_h;                 // internal-order unit face centres (3 planes)
  std::vector<double> dacc_rate, dacc_tilt;  // d profile / d (rate, tilt), per internal face
  std::vector<void*> allocs;
  std::vector<size_t> alloc_bytes;
  size_t bytes = 0;
  double* d_acc = nullptr;
  double* d_dacc = nullptr;
  DevState S{};
  TlmTangents T{};
  double* d_stage = nullptr;
  double* h_stage = nullptr;
  // forward record
  int n_steps = 0;
  bool have_forward = false;
  double dt0 = 0.0;
  std::vector<double> dts_h;
  double* d_dts = nullptr;
  int dts_cap = 0;
  double* d_ck = nullptr;
  int ck_cap = 0;
  // tape of K steps + reverse scratch
  double *tU = nullptr, *tW0 = nullptr, *tU1 = nullptr, *tW1 = nullptr, *tP0 = nullptr, *tP1 = nullptr;
  double *tJ0 = nullptr, *tJ1 = nullptr;
  uint8_t* tmask = nullptr;
  double *d_lam = nullptr, *d_scrU = nullptr, *d_scrW = nullptr;
  AdjScratch X{};
  unsigned err_bits = 0;
  float ms_forward = 0.f, ms_backward = 0.f, ms_tlm = 0.f, ms_frozen = 0.f;
  // branch tape of the branch-frozen forward (validation)
  uint32_t* d_btape = nullptr;
  size_t btape_cap = 0;  // words
  int btape_steps = 0;
  uint32_t* d_bpos = nullptr;
  unsigned* d_berr = nullptr;

  ~Adjoint() {
    if (base) cudaSetDevice(base->device);
    for (void* p : allocs) cudaFree(p);
    if (h_stage) cudaFreeHost(h_stage);
  }

  template <typename T_>
  T_* dalloc(size_t n) {
    void* p = nullptr;
    const size_t b = n * sizeof(T_) > 0 ? n * sizeof(T_) : 16;
    if (cudaMalloc(&p, b) != cudaSuccess) throw std::bad_alloc();
    allocs.push_back(p);
    alloc_bytes.push_back(b);
    bytes += b;
    return static_cast<T_*>(p);
  }
  void dfree(void* p) {
    auto it = std::find(allocs.begin(), allocs.end(), p);
    if (it != allocs.end()) {
      cudaFree(p);
      const size_t i = (size_t)(it - allocs.begin());
      bytes -= alloc_bytes[i];
      alloc_bytes.erase(alloc_bytes.begin() + i);
      allocs.erase(it);
    }
  }
  StepTape tape(int m) const {
    StepTape t;
    t.U = tU + (size_t)m * FS;
    t.W0 = tW0 + (size_t)m * FS;
    t.U1 = tU1 + (size_t)m * FS;
    t.W1 = tW1 + (size_t)m * FS;
    t.P0 = tP0 + (size_t)m * kDim * PS;
    t.P1 = tP1 + (size_t)m * kDim * PS;
    t.J0 = tJ0 + (size_t)m * kTapeJ * PS;
    t.J1 = tJ1 + (size_t)m * kTapeJ * PS;
    t.mask = tmask + (size_t)m * fpad;
    return t;
  }
  cudaStream_t stream() const { return base->stream; }

  void set_theta(const double* theta) {
    par = base->par;
    if (theta) {
      par.accretion_rate = theta[0];
      par.tilt_angle = theta[1];
      par.omega_acc_abs = theta[2];
    }
    P.omega_acc_x = 0;
    P.omega_acc_y = std::sin(par.tilt_angle) * par.omega_acc_abs;
    P.omega_acc_z = std::cos(par.tilt_angle) * par.omega_acc_abs;
    P.acc_rate = par.accretion_rate;
    derive_params(P);
  }
  int upload_profile(const double* dtheta) {
    const std::vector<double> acc = accretion_source_fcn(fcn_h, n_faces, fpad, par, base->area_coeff,
                                                         base->accretion_on, &dacc_rate, &dacc_tilt);
    ADJ_CUDA(cudaMemcpy(d_acc, acc.data(), fpad * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<double> dacc(fpad, 0.0);
    if (dtheta)
      for (int i = 0; i < n_faces; ++i) dacc[i] = dacc_rate[i] * dtheta[0] + dacc_tilt[i] * dtheta[1];
    ADJ_CUDA(cudaMemcpy(d_dacc, dacc.data(), fpad * sizeof(double), cudaMemcpyHostToDevice));
    return SPLASH_OK;
  }
  // reference-order [F][5] host array -> planes (through the pinned stage)
  int to_planes(const double* aos, double* planes) {
    std::memcpy(h_stage, aos, (size_t)n_faces * kDim * sizeof(double));
    ADJ_CUDA(cudaMemcpyAsync(d_stage, h_stage, (size_t)n_faces * kDim * sizeof(double), cudaMemcpyHostToDevice,
                             stream()));
    ADJ_CUDA(fp64_scatter_state(d_stage, base->d_iperm, planes, n_faces, fpad, stream()));
    ADJ_CUDA(cudaStreamSynchronize(stream()));
    return SPLASH_OK;
  }
  int from_planes(const double* planes, double* aos) {
    ADJ_CUDA(fp64_gather_state(planes, base->d_iperm, d_stage, n_faces, fpad, stream()));
    ADJ_CUDA(cudaMemcpyAsync(h_stage, d_stage, (size_t)n_faces * kDim * sizeof(double), cudaMemcpyDeviceToHost,
                             stream()));
    ADJ_CUDA(cudaStreamSynchronize(stream()));
    std::memcpy(aos, h_stage, (size_t)n_faces * kDim * sizeof(double));
    return SPLASH_OK;
  }
  // the initial total mass of the reference constructor (adiabatic.hpp:70-90)
  double total_mass(const double* U_ref) const {
    double tm = 0;
    for (int n = 0; n < n_faces; ++n) tm += U_ref[(size_t)n * kDim] * base->wr_area[n];
    return tm;
  }
  int ensure_capacity(int n) {
    const int nck = (n + K - 1) / K;
    if (n > dts_cap) {
      if (d_dts) dfree(d_dts);
      d_dts = dalloc<double>(n);
      dts_cap = n;
    }
    if (nck > ck_cap) {
      if (d_ck) dfree(d_ck);
      d_ck = dalloc<double>((size_t)nck * FS);
      ck_cap = nck;
    }
    return SPLASH_OK;
  }
  int read_err() {
    unsigned e[4] = {0, 0, 0, 0};
    ADJ_CUDA(cudaMemcpy(e, S.err, sizeof e, cudaMemcpyDeviceToHost));
    err_bits = e[0];
    return SPLASH_OK;
  }

  int forward(const double* U0, const double* theta, int n, double dt0_, double* U_final);
  int backward(const double* lam_final, double* grad_U0, double* grad_theta);
  int tlm(const double* U0, const double* theta, const double* dU0, const double* dtheta, int n, double dt0_,
          double* U_final, double* dU_final);
  int frozen_forward(const double* U0, const double* theta, int n, int record, double* U_final, int64_t* flips);
};

int Adjoint::forward(const double* U0, const double* theta, int n, double dt0_, double* U_final) {
  if (n <= 0) return set_error(SPLASH_E_INVALID, "n_steps must be > 0");
  have_forward = false;
  set_theta(theta);
  int rc = upload_profile(nullptr);
  if (rc) return rc;
  P.total_mass = total_mass(U0);
  derive_params(P);
  try {
    rc = ensure_capacity(n);
  } catch (const std::bad_alloc&) {
    return set_error(SPLASH_E_NOMEM, "device allocation of %d checkpoints failed", (n + K - 1) / K);
  }
  if (rc) return rc;
  rc = to_planes(U0, S.U);
  if (rc) return rc;
  const cudaStream_t st = stream();
  ADJ_CUDA(cudaMemsetAsync(S.err, 0, 4 * sizeof(unsigned), st));
  ADJ_CUDA(cudaMemsetAsync(S.scal, 0, kScCount * sizeof(double), st));
  ADJ_CUDA(fp64_prepare(G, S, P, st));
  ADJ_CUDA(fp64_set_dt0(S, dt0_, st));
  cudaEvent_t e0, e1;
  ADJ_CUDA(cudaEventCreate(&e0));
  ADJ_CUDA(cudaEventCreate(&e1));
  ADJ_CUDA(cudaEventRecord(e0, st));
  for (int i = 0; i < n; ++i) {
    if (i % K == 0)
      ADJ_CUDA(cudaMemcpyAsync(d_ck + (size_t)(i / K) * FS, S.U, FS * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ADJ_CUDA(fp64_step(G, S, P, st));
    ADJ_CUDA(cudaMemcpyAsync(d_dts + i, S.scal + kScDt, sizeof(double), cudaMemcpyDeviceToDevice, st));
  }
  ADJ_CUDA(cudaEventRecord(e1, st));
  ADJ_CUDA(cudaEventSynchronize(e1));
  ADJ_CUDA(cudaEventElapsedTime(&ms_forward, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dts_h.assign(n, 0.0);
  ADJ_CUDA(cudaMemcpy(dts_h.data(), d_dts, n * sizeof(double), cudaMemcpyDeviceToHost));
  rc = read_err();
  if (rc) return rc;
  n_steps = n;
  dt0 = dt0_;
  have_forward = true;
  if (U_final) return from_planes(S.U, U_final);
  return SPLASH_OK;
}

int Adjoint::backward(const double* lam_final, double* grad_U0, double* grad_theta) {
  if (!have_forward) return set_error(SPLASH_E_INVALID, "backward needs a forward run first");
  int rc = to_planes(lam_final, d_lam);
  if (rc) return rc;
  const cudaStream_t st = stream();
  ADJ_CUDA(cudaMemsetAsync(X.th, 0, FS * sizeof(double), st));
  cudaEvent_t e0, e1;
  ADJ_CUDA(cudaEventCreate(&e0));
  ADJ_CUDA(cudaEventCreate(&e1));
  ADJ_CUDA(cudaEventRecord(e0, st));
  const int n_int = (n_steps + K - 1) / K;
  for (int iv = n_int - 1; iv >= 0; --iv) {
    const int c = iv * K;
    const int len = std::min(K, n_steps - c);
    // recompute the interval from its checkpoint, keeping every step's tape
    ADJ_CUDA(cudaMemcpyAsync(tU, d_ck + (size_t)iv * FS, FS * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ADJ_CUDA(rc_prim(G, P, tU, tW0, st));
    for (int m = 0; m < len; ++m) {
      const bool last = (m + 1 == len);
      ADJ_CUDA(rc_step(G, P, d_dts + c + m, tape(m), last ? d_scrU : tU + (size_t)(m + 1) * FS,
                       last ? d_scrW : tW0 + (size_t)(m + 1) * FS, st));
    }
    // reverse steps back to the interval start
    for (int m = len - 1; m >= 0; --m) ADJ_CUDA(adj_step(G, P, dts_h[c + m], tape(m), X, d_lam, st));
  }
  ADJ_CUDA(cudaEventRecord(e1, st));
  ADJ_CUDA(cudaEventSynchronize(e1));
  ADJ_CUDA(cudaEventElapsedTime(&ms_backward, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  rc = read_err();
  if (rc) return rc;
  // parameter adjoints: per-face accumulators -> theta and total mass
  std::vector<double> th(FS);
  ADJ_CUDA(cudaMemcpy(th.data(), X.th, FS * sizeof(double), cudaMemcpyDeviceToHost));
  double s_rate = 0, s_tilt = 0, s_oy = 0, s_oz = 0, s_ar = 0, s_tm = 0;
  for (int f = 0; f < n_faces; ++f) {
    s_rate += th[f] * dacc_rate[f];
    s_tilt += th[f] * dacc_tilt[f];
    s_oy += th[(size_t)fpad + f];
    s_oz += th[2 * (size_t)fpad + f];
    s_ar += th[3 * (size_t)fpad + f];
    s_tm += th[4 * (size_t)fpad + f];
  }
  if (grad_theta) {
    const double st_ = std::sin(par.tilt_angle), ct = std::cos(par.tilt_angle), om = par.omega_acc_abs;
    grad_theta[0] = s_rate + s_ar;
    grad_theta[1] = s_tilt + s_oy * (ct * om) - s_oz * (st_ * om);
    grad_theta[2] = s_oy * st_ + s_oz * ct;
  }
  if (grad_U0) {
    rc = from_planes(d_lam, grad_U0);
    if (rc) return rc;
    // the initial total mass is sum_n U0[n][0] area[n]
    if (s_tm != 0.0)
      for (int f = 0; f < n_faces; ++f) grad_U0[(size_t)f * kDim] += s_tm * base->wr_area[f];
  }
  return SPLASH_OK;
}

int Adjoint::tlm(const double* U0, const double* theta, const double* dU0, const double* dtheta, int n,
                 double dt0_, double* U_final, double* dU_final) {
  if (n <= 0) return set_error(SPLASH_E_INVALID, "n_steps must be > 0");
  set_theta(theta);
  int rc = upload_profile(dtheta);
  if (rc) return rc;
  P.total_mass = total_mass(U0);
  derive_params(P);
  T.d_total_mass = dU0 ? total_mass(dU0) : 0.0;
  const double st_ = std::sin(par.tilt_angle), ct = std::cos(par.tilt_angle), om = par.omega_acc_abs;
  const double dr = dtheta ? dtheta[0] : 0.0, dti = dtheta ? dtheta[1] : 0.0, dom = dtheta ? dtheta[2] : 0.0;
  T.d_omega_y = ct * om * dti + st_ * dom;
  T.d_omega_z = -st_ * om * dti + ct * dom;
  T.d_rate = dr;
  rc = to_planes(U0, S.U);
  if (rc) return rc;
  const cudaStream_t st = stream();
  if (dU0) {
    rc = to_planes(dU0, T.dU);
    if (rc) return rc;
  } else {
    ADJ_CUDA(cudaMemsetAsync(T.dU, 0, FS * sizeof(double), st));
  }
  ADJ_CUDA(cudaMemsetAsync(S.err, 0, 4 * sizeof(unsigned), st));
  ADJ_CUDA(cudaMemsetAsync(S.scal, 0, kScCount * sizeof(double), st));
  ADJ_CUDA(tlm_prepare(G, S, T, P, st));
  ADJ_CUDA(fp64_set_dt0(S, dt0_, st));
  cudaEvent_t e0, e1;
  ADJ_CUDA(cudaEventCreate(&e0));
  ADJ_CUDA(cudaEventCreate(&e1));
  ADJ_CUDA(cudaEventRecord(e0, st));
  for (int i = 0; i < n; ++i) ADJ_CUDA(tlm_step(G, S, T, P, st));
  ADJ_CUDA(cudaEventRecord(e1, st));
  ADJ_CUDA(cudaEventSynchronize(e1));
  ADJ_CUDA(cudaEventElapsedTime(&ms_tlm, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  rc = read_err();
  if (rc) return rc;
  if (U_final) {
    rc = from_planes(S.U, U_final);
    if (rc) return rc;
  }
  if (dU_final) return from_planes(T.dU, dU_final);
  return SPLASH_OK;
}

// The FP64 forward on the dt schedule of the last forward run, with every
// branch decision recorded (mode 1), replayed from the recording (mode 0)
// or compared with it (mode 2).
int Adjoint::frozen_forward(const double* U0, const double* theta, int n, int mode_in, double* U_final,
                            int64_t* flips) {
  if (n <= 0) return set_error(SPLASH_E_INVALID, "n_steps must be > 0");
  if (mode_in < 0 || mode_in > 2) return set_error(SPLASH_E_INVALID, "mode must be 0, 1 or 2");
  const bool record = mode_in == 1;
  const int tmode = record ? 0 : (mode_in == 0 ? 1 : 2);  // taped.cuh: kRecord, kReplay, kCompare
  if (!have_forward || n > n_steps)
    return set_error(SPLASH_E_INVALID,
                     "the branch-frozen forward runs on the dt schedule of a forward run of at least "
                     "n_steps steps: call splash_adjoint_forward first");
  if (!record && n > btape_steps)
    return set_error(SPLASH_E_INVALID, "no branch tape of %d steps: record one first (mode 1)", n);
  set_theta(theta);
  int rc = upload_profile(nullptr);
  if (rc) return rc;
  P.total_mass = total_mass(U0);
  derive_params(P);
  const size_t RW = (size_t)n_faces * taped_words_per_face();
  const size_t need = RW * (1 + 4 * (size_t)n);
  try {
    if (record && need > btape_cap) {
      if (d_btape) dfree(d_btape);
      d_btape = nullptr;
      btape_cap = 0;
      btape_steps = 0;
      d_btape = dalloc<uint32_t>(need);
      btape_cap = need;
    }
    if (!d_bpos) d_bpos = dalloc<uint32_t>(fpad);
    if (!d_berr) d_berr = dalloc<unsigned>(4);
  } catch (const std::bad_alloc&) {
    return set_error(SPLASH_E_NOMEM, "device allocation of the branch tape (%zu bytes) failed",
                     need * sizeof(uint32_t));
  }
  rc = to_planes(U0, S.U);
  if (rc) return rc;
  const cudaStream_t st = stream();
  ADJ_CUDA(cudaMemsetAsync(d_berr, 0, 4 * sizeof(unsigned), st));
  if (record) {
    btape_steps = 0;
    ADJ_CUDA(cudaMemsetAsync(d_btape, 0, need * sizeof(uint32_t), st));
  }
  cudaEvent_t e0, e1;
  ADJ_CUDA(cudaEventCreate(&e0));
  ADJ_CUDA(cudaEventCreate(&e1));
  ADJ_CUDA(cudaEventRecord(e0, st));
  ADJ_CUDA(taped_prim(G, P, S.U, S.W0, d_btape, d_bpos, d_berr, tmode, st));
  for (int i = 0; i < n; ++i)
    ADJ_CUDA(taped_step(G, P, d_dts + i, S.U, S.W0, S.W1, S.uplus, d_scrU, d_btape + RW * (1 + 4 * (size_t)i), d_bpos,
                        d_berr, tmode, st));
  ADJ_CUDA(cudaEventRecord(e1, st));
  ADJ_CUDA(cudaEventSynchronize(e1));
  ADJ_CUDA(cudaEventElapsedTime(&ms_frozen, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  unsigned berr[4] = {0, 0, 0, 0};
  ADJ_CUDA(cudaMemcpy(berr, d_berr, sizeof berr, cudaMemcpyDeviceToHost));
  if (berr[0] & 1u)
    return set_error(SPLASH_E_UNSUPPORTED, "a face made more branch decisions in one launch than its tape slice holds");
  if (berr[0] & 2u)
    return set_error(SPLASH_E_INVALID, "the replay asked for branch decisions the recording does not hold");
  if (flips) {
    unsigned long long f = 0;
    std::memcpy(&f, berr + 2, sizeof f);
    *flips = (int64_t)f;
  }
  if (record) btape_steps = n;
  if (U_final) return from_planes(S.U, U_final);
  return SPLASH_OK;
}

}  // namespace splash

// ============================ C ABI ======================================
using splash::Adjoint;

extern "C" {

int splash_adjoint_create(splash_solver* base_h, int checkpoint_every, splash_adjoint** out) {
  if (!out) return splash::set_error(SPLASH_E_INVALID, "out is NULL");
  *out = nullptr;
  splash::Solver* base = reinterpret_cast<splash::Solver*>(base_h);
  if (!base) return splash::set_error(SPLASH_E_INVALID, "base solver is NULL");
  if (base->precision != SPLASH_PREC_FP64)
    return splash::set_error(SPLASH_E_UNSUPPORTED, "the adjoint differentiates the FP64 step: create the base "
                                                   "solver with SPLASH_PREC_FP64");
  if (base->dim != splash::kDim)
    return splash::set_error(SPLASH_E_UNSUPPORTED, "the adjoint differentiates the adiabatic (dim 5) step");
  if (checkpoint_every <= 0) return splash::set_error(SPLASH_E_INVALID, "checkpoint_every must be > 0");
  if (cudaSetDevice(base->device) != cudaSuccess) return splash::set_error(SPLASH_E_CUDA, "cudaSetDevice failed");
  std::unique_ptr<Adjoint> a(new (std::nothrow) Adjoint());
  if (!a) return splash::set_error(SPLASH_E_NOMEM, "host allocation failed");
  try {
    a->base = base;
    a->K = checkpoint_every;
    a->n_faces = base->n_faces;
    a->fpad = base->fpad;
    a->max_slots = base->max_slots;
    a->PS = (size_t)base->max_slots * base->fpad;
    a->FS = (size_t)splash::kDim * base->fpad;
    a->G = base->G;
    a->P = base->P;
    a->par = base->par;
    const size_t fp = a->fpad, PS = a->PS, FS = a->FS;
    // host copies of the geometry the adjoint needs
    a->fcn_h.assign(3 * fp, 0.0);
    std::vector<int> sten(4 * PS);
    std::vector<int8_t> nsl(fp);
    if (cudaMemcpy(a->fcn_h.data(), base->G.fcn, 3 * fp * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(sten.data(), base->G.sten, 4 * PS * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(nsl.data(), base->G.nslots, fp, cudaMemcpyDeviceToHost) != cudaSuccess)
      return splash::set_error(SPLASH_E_CUDA, "geometry download failed");
    // inverse stencil: for every face, the (slot, position) pairs whose
    // interpolants read it, in slot-plane order
    if (4 * PS > (size_t)INT32_MAX) return splash::set_error(SPLASH_E_UNSUPPORTED, "mesh too large for the adjoint");
    std::vector<int> cnt(fp + 1, 0);
    for (int f = 0; f < a->n_faces; ++f)
      for (int j = 0; j < nsl[f]; ++j)
        for (int p = 0; p < 4; ++p) cnt[sten[p * PS + (size_t)j * fp + f] + 1]++;
    for (size_t i = 0; i < fp; ++i) cnt[i + 1] += cnt[i];
    std::vector<int> ent(cnt[fp]), fill(cnt.begin(), cnt.end() - 1);
    for (size_t s = 0; s < PS; ++s) {
      const int f = (int)(s % fp), j = (int)(s / fp);
      if (f >= a->n_faces || j >= nsl[f]) continue;
      for (int p = 0; p < 4; ++p) ent[fill[sten[p * PS + s]]++] = (int)(s * 4 + p);
    }
    int* d_off = a->dalloc<int>(fp + 1);
    int* d_ent = a->dalloc<int>(ent.size());
    if (cudaMemcpy(d_off, cnt.data(), (fp + 1) * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d_ent, ent.data(), ent.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
      return splash::set_error(SPLASH_E_CUDA, "inverse stencil upload failed");
    a->d_acc = a->dalloc<double>(fp);
    a->d_dacc = a->dalloc<double>(fp);
    a->G.acc_src = a->d_acc;
    // value state and tangents
    splash::DevState& S = a->S;
    S.U = a->dalloc<double>(FS);
    S.W0 = a->dalloc<double>(FS);
    S.W1 = a->dalloc<double>(FS);
    S.uplus = a->dalloc<double>(splash::kDim * PS);
    S.partial = a->dalloc<double>((size_t)splash::fp64_partial_blocks(a->n_faces) * splash::kPartialStride);
    S.scal = a->dalloc<double>(splash::kScCount);
    S.err = a->dalloc<unsigned int>(4);
    a->T.dU = a->dalloc<double>(FS);
    a->T.dW0 = a->dalloc<double>(FS);
    a->T.dW1 = a->dalloc<double>(FS);
    a->T.duplus = a->dalloc<double>(splash::kDim * PS);
    a->T.dacc = a->d_dacc;
    // tape of K steps
    const size_t K = a->K;
    a->tU = a->dalloc<double>(K * FS);
    a->tW0 = a->dalloc<double>(K * FS);
    a->tU1 = a->dalloc<double>(K * FS);
    a->tW1 = a->dalloc<double>(K * FS);
    a->tP0 = a->dalloc<double>(K * splash::kDim * PS);
    a->tP1 = a->dalloc<double>(K * splash::kDim * PS);
    a->tJ0 = a->dalloc<double>(K * splash::kTapeJ * PS);
    a->tJ1 = a->dalloc<double>(K * splash::kTapeJ * PS);
    a->tmask = a->dalloc<uint8_t>(K * fp);
    a->d_lam = a->dalloc<double>(FS);
    a->d_scrU = a->dalloc<double>(FS);
    a->d_scrW = a->dalloc<double>(FS);
    splash::AdjScratch& X = a->X;
    X.A = a->dalloc<double>(splash::kDim * PS);
    X.B = a->dalloc<double>(splash::kDim * PS);
    X.PU = a->dalloc<double>(2 * splash::kDim * PS);
    X.Lw = a->dalloc<double>(FS);
    X.la2 = a->dalloc<double>(FS);
    X.la1 = a->dalloc<double>(FS);
    X.lam1 = a->dalloc<double>(FS);
    X.th = a->dalloc<double>(FS);
    X.inv_off = d_off;
    X.inv_ent = d_ent;
    a->d_stage = a->dalloc<double>((size_t)a->n_faces * splash::kDim);
    if (cudaMallocHost(&a->h_stage, (size_t)a->n_faces * splash::kDim * sizeof(double)) != cudaSuccess)
      return splash::set_error(SPLASH_E_NOMEM, "pinned staging allocation failed");
  } catch (const std::bad_alloc&) {
    return splash::set_error(SPLASH_E_NOMEM, "device allocation failed (tape of %d steps)", checkpoint_every);
  }
  *out = reinterpret_cast<splash_adjoint*>(a.release());
  return SPLASH_OK;
}

int splash_adjoint_destroy(splash_adjoint* h) {
  delete reinterpret_cast<Adjoint*>(h);
  return SPLASH_OK;
}

#define GET_ADJ(h)                                                                  \
  Adjoint* a = reinterpret_cast<Adjoint*>(h);                                       \
  if (!a) return splash::set_error(SPLASH_E_INVALID, "adjoint handle is NULL");    \
  if (cudaSetDevice(a->base->device) != cudaSuccess)                                \
  return splash::set_error(SPLASH_E_CUDA, "cudaSetDevice failed")

int splash_adjoint_forward(splash_adjoint* h, const double* U0, const double* theta, int n_steps, double dt0,
                           double* U_final) {
  GET_ADJ(h);
  if (!U0) return splash::set_error(SPLASH_E_INVALID, "U0 is NULL");
  return a->forward(U0, theta, n_steps, dt0, U_final);
}

int splash_adjoint_backward(splash_adjoint* h, const double* lambda_final, double* grad_U0, double* grad_theta) {
  GET_ADJ(h);
  if (!lambda_final) return splash::set_error(SPLASH_E_INVALID, "lambda_final is NULL");
  return a->backward(lambda_final, grad_U0, grad_theta);
}

int splash_adjoint_run(splash_adjoint* h, const double* U0, const double* theta, int n_steps, double dt0,
                       const double* sigma_target, double* loss, double* grad_U0, double* grad_theta) {
  GET_ADJ(h);
  if (!U0 || !sigma_target) return splash::set_error(SPLASH_E_INVALID, "U0 and sigma_target must be non-NULL");
  const size_t n = (size_t)a->n_faces;
  std::vector<double> U(n * splash::kDim), lam(n * splash::kDim, 0.0);
  int rc = a->forward(U0, theta, n_steps, dt0, U.data());
  if (rc) return rc;
  // loss = 1/2 sum_n area_n (Sigma_n - Sigma*_n)^2, reference face order
  double L = 0.0;
  for (size_t i = 0; i < n; ++i) {
    const double d = U[i * splash::kDim] - sigma_target[i];
    L += 0.5 * a->base->wr_area[i] * d * d;
    lam[i * splash::kDim] = a->base->wr_area[i] * d;
  }
  if (loss) *loss = L;
  return a->backward(lam.data(), grad_U0, grad_theta);
}

int splash_tlm_run(splash_adjoint* h, const double* U0, const double* theta, const double* dU0,
                   const double* dtheta, int n_steps, double dt0, double* U_final, double* dU_final) {
  GET_ADJ(h);
  if (!U0) return splash::set_error(SPLASH_E_INVALID, "U0 is NULL");
  return a->tlm(U0, theta, dU0, dtheta, n_steps, dt0, U_final, dU_final);
}

int splash_adjoint_branch_tape(splash_adjoint* h, const double* U0, const double* theta, int n_steps, int mode,
                               double* U_final, int64_t* count) {
  GET_ADJ(h);
  if (!U0) return splash::set_error(SPLASH_E_INVALID, "U0 is NULL");
  return a->frozen_forward(U0, theta, n_steps, mode, U_final, count);
}

int splash_adjoint_info(splash_adjoint* h, double out[8]) {
  GET_ADJ(h);
  if (!out) return splash::set_error(SPLASH_E_INVALID, "out is NULL");
  int clipped = 0;
  double dmin = 0, dmax = 0;
  if (!a->dts_h.empty()) {
    dmin = *std::min_element(a->dts_h.begin(), a->dts_h.end());
    dmax = *std::max_element(a->dts_h.begin(), a->dts_h.end());
    for (double d : a->dts_h)
      if (d < a->dt0) ++clipped;
  }
  out[0] = a->n_steps;
  out[1] = clipped;
  out[2] = dmin;
  out[3] = dmax;
  out[4] = a->ms_forward;
  out[5] = a->ms_backward;
  out[6] = a->ms_tlm;
  out[7] = (double)a->bytes;
  return SPLASH_OK;
}

int splash_adjoint_error_word(splash_adjoint* h, unsigned* err) {
  GET_ADJ(h);
  if (!err) return splash::set_error(SPLASH_E_INVALID, "err is NULL");
  *err = a->err_bits;
  return SPLASH_OK;
}

int splash_adjoint_dt_schedule(splash_adjoint* h, double* dts, int n) {
  GET_ADJ(h);
  if (!dts || n < a->n_steps) return splash::set_error(SPLASH_E_INVALID, "dts must hold n_steps values");
  std::copy(a->dts_h.begin(), a->dts_h.end(), dts);
  return SPLASH_OK;
}

}  // extern "C"
