// results.cu -- DADF5 result files and restart files of an RVE (host side).
//
// Results follow the layout DAMASK writes (reference src/result.f90:80-160,
// phase_mechanical.f90:919-985, discretization.f90:102-116, grid geometry
// attributes): root attributes DADF5_version_major/minor, creator, created, call;
// /geometry {cells, size, origin}; /cell_to/{phase, homogenization} as
// {label (space-padded string), entry (int64)} records; /setup with the input files; and per written increment
// /increment_<n> {t/s} with geometry/{u_n, u_p},
// phase/<phase>/mechanical/{F, F_e, F_p, L_p, O, P, xi_sl} and
// homogenization/<homogenization>/mechanical.  Datasets carry description, unit
// and creator attributes; tensors are (cells, 3, 3) row-major [cell][i][j].
// The orientation O is the quaternion of the rotational part of F_e, transposed
// (phase.f90:590; math.f90:1117-1156 closed-form polar decomposition;
// rotations.f90:518-546 matrix -> quaternion with P = -1).
//
// Restart files hold everything an RVE needs to continue a load case exactly
// where it stopped (the reference's restart: materialpoint.f90:163-202,
// phase_mechanical.f90:1264-1298 and the grid solver's F, F_lastInc, F_aim and
// averaged stiffness): per-point state planes, the solution and rate fields, and
// the solver's host state.  A continued run is bitwise identical to an
// uninterrupted one.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "h5lite.hpp"
#include "rve.cuh"

using namespace dgx;

namespace {

void rotational_part(const double F[9], double R[9]) {
  auto clip = [](double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); };
  double C[9], FF[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double c = 0.0, f = 0.0;
      for (int k = 0; k < 3; ++k) { c += F[k + 3 * i] * F[k + 3 * j]; f += F[i + 3 * k] * F[k + 3 * j]; }
      C[i + 3 * j] = c; FF[i + 3 * j] = f;
    }
  // invariants of C and F, principal stretches from the trigonometric cubic solution
  const double I1 = C[0] + C[4] + C[8];
  const double I2 = C[0] * C[4] + C[4] * C[8] + C[8] * C[0] - C[3] * C[3] - C[7] * C[7] - C[6] * C[6];
  const double I3 = C[0] * (C[4] * C[8] - C[7] * C[5]) - C[3] * (C[1] * C[8] - C[7] * C[2]) +
                    C[6] * (C[1] * C[5] - C[4] * C[2]);
  const double trF = F[0] + F[4] + F[8], trFF = FF[0] + FF[4] + FF[8];
  const double IF1 = trF, IF2 = 0.5 * (trF * trF - trFF);
  const double x = std::pow(clip(I1 * I1 - 3.0 * I2, 0.0, INFINITY), 1.5);
  double lam[3];
  if (x != 0.0) {
    const double Phi = std::acos(clip((I1 * I1 * I1 - 4.5 * I1 * I2 + 13.5 * I3) / x, -1.0, 1.0));
    for (int k = 0; k < 3; ++k) {
      double l = I1 + (2.0 * std::sqrt(clip(I1 * I1 - 3.0 * I2, 0.0, INFINITY))) *
                 std::cos((Phi - 6.283185307179586476925286766559 * (k + 1.0)) / 3.0);
      lam[k] = std::sqrt(clip(l, 0.0, INFINITY) / 3.0);
    }
  } else {
    for (int k = 0; k < 3; ++k) lam[k] = std::sqrt(I1 / 3.0);
  }
  const double IU1 = lam[0] + lam[1] + lam[2];
  const double IU2 = lam[0] * lam[1] + lam[1] * lam[2] + lam[2] * lam[0];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double FC = 0.0;
      for (int k = 0; k < 3; ++k) FC += F[i + 3 * k] * C[k + 3 * j];
      R[i + 3 * j] = (i == j ? IU1 * IF2 : 0.0) + (IU1 * IU1 - IU2) * F[i + 3 * j] - IU1 * IF1 * F[j + 3 * i] +
                     IU1 * FF[j + 3 * i] - FC;
    }
  const double d = R[0] * (R[4] * R[8] - R[7] * R[5]) - R[3] * (R[1] * R[8] - R[7] * R[2]) +
                   R[6] * (R[1] * R[5] - R[4] * R[2]);
  const double s = std::pow(d, -1.0 / 3.0);
  for (int k = 0; k < 9; ++k) R[k] *= s;
}

void matrix_to_quaternion(const double* om, double* q) {
  auto M = [&](int i, int j) { return om[(i - 1) + 3 * (j - 1)]; };
  const double tr = M(1, 1) + M(2, 2) + M(3, 3);
  double s;
  if (tr > 0.0) {
    s = 0.5 / std::sqrt(tr + 1.0);
    q[0] = 0.25 / s; q[1] = (M(3, 2) - M(2, 3)) * s; q[2] = (M(1, 3) - M(3, 1)) * s; q[3] = (M(2, 1) - M(1, 2)) * s;
  } else if (M(1, 1) > M(2, 2) && M(1, 1) > M(3, 3)) {
    s = 2.0 * std::sqrt(1.0 + M(1, 1) - M(2, 2) - M(3, 3));
    q[0] = (M(3, 2) - M(2, 3)) / s; q[1] = 0.25 * s; q[2] = (M(1, 2) + M(2, 1)) / s; q[3] = (M(1, 3) + M(3, 1)) / s;
  } else if (M(2, 2) > M(3, 3)) {
    s = 2.0 * std::sqrt(1.0 + M(2, 2) - M(1, 1) - M(3, 3));
    q[0] = (M(1, 3) - M(3, 1)) / s; q[1] = (M(1, 2) + M(2, 1)) / s; q[2] = 0.25 * s; q[3] = (M(2, 3) + M(3, 2)) / s;
  } else {
    s = 2.0 * std::sqrt(1.0 + M(3, 3) - M(1, 1) - M(2, 2));
    q[0] = (M(2, 1) - M(1, 2)) / s; q[1] = (M(1, 3) + M(3, 1)) / s; q[2] = (M(2, 3) + M(3, 2)) / s; q[3] = 0.25 * s;
  }
  if (std::copysign(1.0, q[0]) < 0.0) for (int k = 0; k < 4; ++k) q[k] = -q[k];
  for (int k = 1; k < 4; ++k) if (q[k] != 0.0) q[k] = -q[k];
  const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int k = 0; k < 4; ++k) q[k] /= n;
}

std::string now_string() {
  char buf[64];
  time_t t = time(nullptr);
  struct tm tmv;
  gmtime_r(&t, &tmv);
  strftime(buf, sizeof(buf), "%Y-%m-%d %H:%M:%S+0000", &tmv);
  return buf;
}

h5lite::Attr a_str(const char* n, const std::string& v) { return h5lite::attr_str(n, v); }

}  // namespace

struct dgx_result {
  h5lite::Writer w;
  std::string phase, homog;
  int cells[3] = {0, 0, 0};
  int64_t N = 0;
};

extern "C" dgx_status dgx_result_open(const char* path, const dgx_rve* r, const char* phase, const char* homogenization,
                                      dgx_result** out) {
  if (!path || !r || !out) return DGX_ERR_ARG;
  dgx_result* res = new dgx_result();
  res->phase = phase && *phase ? phase : "phase";
  res->homog = homogenization && *homogenization ? homogenization : "SX";
  for (int i = 0; i < 3; ++i) res->cells[i] = r->cells[i];
  res->N = r->N;
  if (!res->w.open(path)) { set_err("dgx_result_open: cannot create %s", path); delete res; return DGX_ERR_ARG; }
  h5lite::Node* root = res->w.root();
  root->attrs.push_back(h5lite::attr_i32("DADF5_version_major", {1}, true));
  root->attrs.push_back(h5lite::attr_i32("DADF5_version_minor", {0}, true));
  root->attrs.push_back(a_str("creator", "solver_cpp_gb300 spectral solver (GB300)"));
  root->attrs.push_back(a_str("created", now_string()));
  root->attrs.push_back(a_str("call", "dgx_result_open"));
  h5lite::Node* geo = res->w.group("geometry");
  geo->attrs.push_back(h5lite::attr_i32("cells", {r->cells[0], r->cells[1], r->cells[2]}));
  geo->attrs.push_back(h5lite::attr_f64("size", {r->geom[0], r->geom[1], r->geom[2]}));
  geo->attrs.push_back(h5lite::attr_f64("origin", {0.0, 0.0, 0.0}));
  // cell_to: one constituent, every cell an entry of the single phase / homogenization
  {
    h5lite::Node* ct = res->w.group("cell_to");
    ct->attrs.push_back(a_str("description", "mappings to place data in space"));
    for (int which = 0; which < 2; ++which) {
      const std::string& label = which == 0 ? res->phase : res->homog;
      const uint32_t L = (uint32_t)label.size();
      std::vector<uint8_t> rec((size_t)r->N * (L + 8), 0);
      for (int64_t e = 0; e < r->N; ++e) {
        memcpy(&rec[(size_t)e * (L + 8)], label.c_str(), label.size());
        int64_t v = e;
        memcpy(&rec[(size_t)e * (L + 8) + L], &v, 8);
      }
      std::vector<uint64_t> dims = which == 0 ? std::vector<uint64_t>{(uint64_t)r->N, 1} : std::vector<uint64_t>{(uint64_t)r->N};
      res->w.dataset(which == 0 ? "cell_to/phase" : "cell_to/homogenization", h5lite::LABEL_ENTRY, dims, rec.data(),
                     rec.size(), L);
    }
  }
  res->w.group("setup")->attrs.push_back(a_str("description", "input data used to run the simulation"));
  *out = res;
  return DGX_OK;
}

extern "C" dgx_status dgx_result_add_setup(dgx_result* res, const char* name, const char* content, int64_t length) {
  if (!res || !name || !content || length < 0) return DGX_ERR_ARG;
  std::string s(content, (size_t)length);
  res->w.dataset(std::string("setup/") + name, h5lite::STR, {}, s.c_str(), s.size() + 1, (uint32_t)s.size() + 1);
  return DGX_OK;
}

extern "C" dgx_status dgx_result_write_increment(dgx_result* res, dgx_rve* r, int32_t inc, double t) {
  if (!res || !r || inc < 0) return DGX_ERR_ARG;
  if (r->in_batch) { set_err("RVE is driven by a batch"); return DGX_ERR_STATE; }
  return result_write_impl(res, r, inc, t);
}

dgx_status dgx::result_write_impl(dgx_result* res, dgx_rve* r, int32_t inc, double t) {
  if (r->cells[0] != res->cells[0] || r->cells[1] != res->cells[1] || r->cells[2] != res->cells[2]) {
    set_err("dgx_result_write_increment: RVE grid differs from the file's"); return DGX_ERR_ARG;
  }
  const int64_t N = r->N;
  const int64_t Nn = (int64_t)(r->cells[0] + 1) * (r->cells[1] + 1) * (r->cells[2] + 1);
  const std::string g = "increment_" + std::to_string(inc);
  res->w.group(g)->attrs.push_back(h5lite::attr_f64("t/s", {t}, true));
  const std::string created = now_string();
  auto tag = [&](h5lite::Node* d, const char* desc, const char* unit) {
    d->attrs.push_back(a_str("creator", "solver_cpp_gb300"));
    d->attrs.push_back(a_str("created", created));
    d->attrs.push_back(a_str("description", desc));
    d->attrs.push_back(a_str("unit", unit));
  };
  // geometry
  std::vector<double> un(3 * Nn), up(3 * N);
  TRY(update_coords_impl(r, un.data(), up.data()));
  tag(res->w.dataset(g + "/geometry/u_n", h5lite::F64, {(uint64_t)Nn, 3}, un.data(), un.size() * 8),
      "displacements of the nodes", "m");
  tag(res->w.dataset(g + "/geometry/u_p", h5lite::F64, {(uint64_t)N, 3}, up.data(), up.size() * 8),
      "displacements of the materialpoints (cell centers)", "m");
  // phase mechanical outputs: library layout (3,3,N) column-major -> [cell][i][j]
  const std::string ph = g + "/phase/" + res->phase + "/mechanical/";
  std::vector<double> buf(9 * N), rowm(9 * N), Fe(9 * N);
  struct Out { const char* field; const char* name; const char* desc; const char* unit; };
  const Out outs[] = {{"F", "F", "deformation gradient", "1"},
                      {"Fe", "F_e", "elastic deformation gradient", "1"},
                      {"Fp", "F_p", "plastic deformation gradient", "1"},
                      {"Lp", "L_p", "plastic velocity gradient", "1/s"},
                      {"P", "P", "first Piola-Kirchhoff stress", "Pa"}};
  for (const Out& o : outs) {
    TRY(dgx_get(r, o.field, buf.data()));
    if (!strcmp(o.field, "Fe")) Fe = buf;
    for (int64_t e = 0; e < N; ++e)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) rowm[9 * e + 3 * i + j] = buf[9 * e + i + 3 * j];
    tag(res->w.dataset(ph + o.name, h5lite::F64, {(uint64_t)N, 3, 3}, rowm.data(), rowm.size() * 8), o.desc, o.unit);
  }
  std::vector<double> O(4 * N);
  for (int64_t e = 0; e < N; ++e) {
    double R[9], Rt[9];
    rotational_part(&Fe[9 * e], R);
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) Rt[i + 3 * j] = R[j + 3 * i];
    matrix_to_quaternion(Rt, &O[4 * e]);
  }
  h5lite::Node* dO = res->w.dataset(ph + "O", h5lite::F64, {(uint64_t)N, 4}, O.data(), O.size() * 8);
  tag(dO, "crystal orientation as quaternion q_0 (q_1 q_2 q_3)", "1");
  dO->attrs.push_back(a_str("lattice", "cF"));
  std::vector<double> xi(12 * N);
  TRY(dgx_get(r, "xi", xi.data()));
  tag(res->w.dataset(ph + "xi_sl", h5lite::F64, {(uint64_t)N, 12}, xi.data(), xi.size() * 8),
      "resistance against plastic slip", "Pa");
  res->w.group(g + "/homogenization/" + res->homog + "/mechanical");
  return DGX_OK;
}

extern "C" dgx_status dgx_result_close(dgx_result* res) {
  if (!res) return DGX_ERR_ARG;
  bool ok = res->w.close();
  delete res;
  if (!ok) { set_err("dgx_result_close: write failed"); return DGX_ERR_STATE; }
  return DGX_OK;
}

// ------------------------------------------------------------------ restart
namespace {

std::vector<std::pair<std::string, double*>> state_planes(dgx_rve* r) {
  return {{"phase/F", r->ps.F},       {"phase/F0", r->ps.F0},  {"phase/F_p0", r->ps.Fp0}, {"phase/L_p0", r->ps.Lp0},
          {"phase/S0", r->ps.S0},     {"phase/F_p", r->ps.Fp}, {"phase/L_p", r->ps.Lp},   {"phase/S", r->ps.S},
          {"phase/F_e", r->ps.Fe},    {"phase/P", r->ps.P},    {"solver/F", r->X},        {"solver/F_lastInc", r->F_last_inc},
          {"solver/F_dot", r->F_dot}};
}

}  // namespace

extern "C" dgx_status dgx_restart_write(dgx_rve* r, const char* path) {
  if (!r || !path) return DGX_ERR_ARG;
  if (r->in_batch) { set_err("RVE is driven by a batch"); return DGX_ERR_STATE; }
  return restart_write_impl(r, path);
}

dgx_status dgx::restart_write_impl(dgx_rve* r, const char* path) {
  if (!r->initialized) { set_err("dgx_restart_write before dgx_solver_init"); return DGX_ERR_STATE; }
  h5lite::Writer w;
  if (!w.open(path)) { set_err("dgx_restart_write: cannot create %s", path); return DGX_ERR_ARG; }
  const int64_t N = r->N;
  w.root()->attrs.push_back(h5lite::attr_i32("cells", {r->cells[0], r->cells[1], r->cells[2]}));
  CK(cudaStreamSynchronize(r->st));
  std::vector<double> buf(24 * N);
  for (auto& p : state_planes(r)) {
    CK(cudaMemcpy(buf.data(), p.second, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost));
    w.dataset(p.first, h5lite::F64, {9, (uint64_t)N}, buf.data(), sizeof(double) * 9 * N);
  }
  CK(cudaMemcpy(buf.data(), r->ps.st0, sizeof(double) * 24 * N, cudaMemcpyDeviceToHost));
  w.dataset("phase/state0", h5lite::F64, {24, (uint64_t)N}, buf.data(), sizeof(double) * 24 * N);
  CK(cudaMemcpy(buf.data(), r->ps.st, sizeof(double) * 24 * N, cudaMemcpyDeviceToHost));
  w.dataset("phase/state", h5lite::F64, {24, (uint64_t)N}, buf.data(), sizeof(double) * 24 * N);
  auto arr = [&](const char* n, const double* v, size_t k) { w.dataset(std::string("solver/") + n, h5lite::F64, {k}, v, 8 * k); };
  arr("F_aim", r->F_aim, 9); arr("F_aim_lastInc", r->F_aim_last_inc, 9); arr("F_aimDot", r->F_aim_dot, 9);
  arr("P_aim", r->P_aim, 9); arr("P_av", r->P_av, 9);
  arr("C_volAvg", r->C_volAvg, 81); arr("C_volAvgLastInc", r->C_volAvgLastInc, 81);
  arr("C_minMaxAvg", r->C_minMaxAvg, 81); arr("C_minMaxAvgLastInc", r->C_minMaxAvgLastInc, 81);
  arr("C_ref", r->C_ref, 81); arr("S", r->S, 81); arr("rot_q", r->rot_q, 4);
  const double sc[8] = {r->delta_t, r->t, r->dt, r->dt_prev, r->t_0, r->tangent_dt, r->err_div, r->err_BC};
  arr("scalars", sc, 8);
  const int32_t iv[6] = {r->cut_back, r->cut_back_level, r->guess, r->cur_step, r->terminally_ill, r->total_iter};
  w.dataset("solver/integers", h5lite::I32, {6}, iv, sizeof(iv));
  w.dataset("solver/stress_mask", h5lite::I32, {9}, r->stress_mask, sizeof(r->stress_mask));
  w.dataset("solver/cells", h5lite::I32, {3}, r->cells, sizeof(r->cells));
  if (!w.close()) { set_err("dgx_restart_write: write failed"); return DGX_ERR_STATE; }
  return DGX_OK;
}

extern "C" dgx_status dgx_restart_read(dgx_rve* r, const char* path) {
  if (!r || !path) return DGX_ERR_ARG;
  if (r->in_batch) { set_err("RVE is driven by a batch"); return DGX_ERR_STATE; }
  h5lite::Reader rd;
  if (!rd.open(path)) { set_err("dgx_restart_read: cannot read %s", path); return DGX_ERR_ARG; }
  const int64_t N = r->N;
  std::vector<uint8_t> b;
  std::vector<uint64_t> dims;
  auto need = [&](const std::string& n, size_t bytes) -> bool {
    if (!rd.read(n, b, &dims) || b.size() != bytes) { set_err("dgx_restart_read: %s missing or of the wrong size", n.c_str()); return false; }
    return true;
  };
  if (!need("solver/cells", 12)) return DGX_ERR_ARG;
  if (memcmp(b.data(), r->cells, 12) != 0) { set_err("dgx_restart_read: restart grid differs from the RVE's"); return DGX_ERR_ARG; }
  CK(cudaStreamSynchronize(r->st));
  for (auto& p : state_planes(r)) {
    if (!need(p.first, sizeof(double) * 9 * N)) return DGX_ERR_ARG;
    CK(cudaMemcpy(p.second, b.data(), b.size(), cudaMemcpyHostToDevice));
  }
  if (!need("phase/state0", sizeof(double) * 24 * N)) return DGX_ERR_ARG;
  CK(cudaMemcpy(r->ps.st0, b.data(), b.size(), cudaMemcpyHostToDevice));
  if (!need("phase/state", sizeof(double) * 24 * N)) return DGX_ERR_ARG;
  CK(cudaMemcpy(r->ps.st, b.data(), b.size(), cudaMemcpyHostToDevice));
  auto arr = [&](const char* n, double* v, size_t k) -> bool {
    if (!need(std::string("solver/") + n, 8 * k)) return false;
    memcpy(v, b.data(), 8 * k);
    return true;
  };
  if (!(arr("F_aim", r->F_aim, 9) && arr("F_aim_lastInc", r->F_aim_last_inc, 9) && arr("F_aimDot", r->F_aim_dot, 9) &&
        arr("P_aim", r->P_aim, 9) && arr("P_av", r->P_av, 9) && arr("C_volAvg", r->C_volAvg, 81) &&
        arr("C_volAvgLastInc", r->C_volAvgLastInc, 81) && arr("C_minMaxAvg", r->C_minMaxAvg, 81) &&
        arr("C_minMaxAvgLastInc", r->C_minMaxAvgLastInc, 81) && arr("C_ref", r->C_ref, 81) && arr("S", r->S, 81) &&
        arr("rot_q", r->rot_q, 4)))
    return DGX_ERR_ARG;
  double sc[8];
  if (!arr("scalars", sc, 8)) return DGX_ERR_ARG;
  r->delta_t = sc[0]; r->t = sc[1]; r->dt = sc[2]; r->dt_prev = sc[3]; r->t_0 = sc[4]; r->tangent_dt = sc[5];
  r->err_div = sc[6]; r->err_BC = sc[7];
  if (!need("solver/integers", 6 * 4)) return DGX_ERR_ARG;
  int32_t iv[6];
  memcpy(iv, b.data(), sizeof(iv));
  r->cut_back = iv[0]; r->cut_back_level = iv[1]; r->guess = iv[2]; r->cur_step = iv[3]; r->terminally_ill = iv[4];
  r->total_iter = iv[5];
  if (!need("solver/stress_mask", 9 * 4)) return DGX_ERR_ARG;
  memcpy(r->stress_mask, b.data(), sizeof(r->stress_mask));
  TRY(set_reference_stiffness(r));
  CK(cudaStreamSynchronize(r->st));
  r->tangent_fresh = false;
  r->initialized = true;
  return DGX_OK;
}
