// A C++ caller of the C ABI that keeps its fields on the device, as a drop-in grid
// solver would: reads a VTI geometry from memory (dgx_vti_read_cells_size_origin /
// dgx_vti_read_dataset_int), creates an RVE, fetches the library-owned device fields
// (dgx_fields), writes F on the device, runs the constitutive response in place
// (dgx_constitutive_response_fields) and checks P and dPdF against the host-copy entry
// point (dgx_constitutive_response) on a second RVE of the same inputs, then commits and
// checks the exported committed F.
// Usage: fields_check <file.vti>; prints "ok" and exits 0 on success.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/dgx.h"

#define REQUIRE(c, ...) do { if (!(c)) { std::printf(__VA_ARGS__); std::printf("\n"); return 1; } } while (0)

static double rel(const std::vector<double>& a, const std::vector<double>& b) {
  double d = 0.0, m = 0.0;
  for (size_t k = 0; k < a.size(); ++k) { d = std::fmax(d, std::fabs(a[k] - b[k])); m = std::fmax(m, std::fabs(b[k])); }
  return m > 0 ? d / m : d;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  std::ifstream f(argv[1], std::ios::binary);
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string vti = ss.str();
  int32_t cells[3];
  double size[3], origin[3];
  REQUIRE(dgx_vti_read_cells_size_origin(vti.data(), (int64_t)vti.size(), cells, size, origin) == DGX_OK,
          "vti header: %s", dgx_last_error());
  const int64_t N = (int64_t)cells[0] * cells[1] * cells[2];
  std::vector<int32_t> mat(N);
  int64_t count = N;
  const char label[] = "material";
  REQUIRE(dgx_vti_read_dataset_int(vti.data(), (int64_t)vti.size(), label, 8, mat.data(), &count) == DGX_OK && count == N,
          "vti dataset: %s", dgx_last_error());
  int32_t nmat = 0;
  for (int32_t m : mat) nmat = m + 1 > nmat ? m + 1 : nmat;
  std::vector<double> q(4 * (size_t)nmat);
  for (int32_t m = 0; m < nmat; ++m) {                      // fixed, distinct unit quaternions
    double a = 0.3 + 0.17 * m, b = 0.2 - 0.05 * m, c = 0.1 * m, d = 1.0;
    double n = std::sqrt(a * a + b * b + c * c + d * d);
    q[4 * m] = d / n; q[4 * m + 1] = a / n; q[4 * m + 2] = b / n; q[4 * m + 3] = c / n;
  }
  dgx_material mp;
  dgx_numerics num;
  dgx_material_default(&mp);
  dgx_numerics_default(&num);
  dgx_rve *dev_rve = nullptr, *host_rve = nullptr;
  REQUIRE(dgx_rve_create(cells, size, mat.data(), nmat, q.data(), &mp, &num, &dev_rve) == DGX_OK, "create: %s",
          dgx_last_error());
  REQUIRE(dgx_rve_create(cells, size, mat.data(), nmat, q.data(), &mp, &num, &host_rve) == DGX_OK, "create: %s",
          dgx_last_error());
  dgx_field_ptrs fp;
  REQUIRE(dgx_fields(dev_rve, 1, &fp) == DGX_OK, "fields: %s", dgx_last_error());
  REQUIRE(fp.n == N && fp.F && fp.F0 && fp.P && fp.dPdF && fp.terminally_ill && fp.stream, "field pointers");
  cudaStream_t st = (cudaStream_t)fp.stream;
  // F0 and F start as the identity (committed F of a fresh RVE)
  std::vector<double> F(9 * N), F0(9 * N);
  REQUIRE(cudaMemcpyAsync(F0.data(), fp.F0, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
          cudaStreamSynchronize(st) == cudaSuccess, "read F0");
  for (int64_t e = 0; e < N; ++e)
    for (int k = 0; k < 9; ++k) REQUIRE(F0[9 * e + k] == ((k % 4) == 0 ? 1.0 : 0.0), "F0 not identity");
  // two load steps: write F on the device, respond in place, compare with the host path
  for (int step = 1; step <= 2; ++step) {
    for (int64_t e = 0; e < N; ++e)
      for (int k = 0; k < 9; ++k)
        F[9 * e + k] = ((k % 4) == 0 ? 1.0 : 0.0) + (k == 0 ? 1e-3 * step : 0.0) + (k == 4 || k == 8 ? -4e-4 * step : 0.0) +
                       2e-5 * std::sin(0.37 * e + k);
    REQUIRE(cudaMemcpyAsync(fp.F, F.data(), sizeof(double) * 9 * N, cudaMemcpyHostToDevice, st) == cudaSuccess,
            "write F");
    REQUIRE(dgx_constitutive_response_fields(dev_rve, 0.5, 0, (int32_t)N, 1) == DGX_OK, "response_fields: %s",
            dgx_last_error());
    std::vector<double> P_dev(9 * N), dP_dev(81 * N), P_host(9 * N), dP_host(81 * N);
    int32_t ill_dev = -1, ill_host = -1;
    REQUIRE(cudaMemcpy(P_dev.data(), fp.P, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost) == cudaSuccess &&
            cudaMemcpy(dP_dev.data(), fp.dPdF, sizeof(double) * 81 * N, cudaMemcpyDeviceToHost) == cudaSuccess &&
            cudaMemcpy(&ill_dev, fp.terminally_ill, sizeof(int32_t), cudaMemcpyDeviceToHost) == cudaSuccess,
            "read results");
    REQUIRE(dgx_constitutive_response(host_rve, F.data(), 0.5, 0, (int32_t)N, P_host.data(), dP_host.data(), &ill_host) ==
            DGX_OK, "response: %s", dgx_last_error());
    REQUIRE(ill_dev == 0 && ill_host == 0, "terminally ill");
    REQUIRE(rel(P_dev, P_host) == 0.0, "P differs: %g", rel(P_dev, P_host));
    REQUIRE(rel(dP_dev, dP_host) == 0.0, "dPdF differs: %g", rel(dP_dev, dP_host));
    double Pa[9], Pb[9];
    REQUIRE(dgx_averages(dev_rve, Pa, nullptr, nullptr) == DGX_OK && dgx_averages(host_rve, Pb, nullptr, nullptr) == DGX_OK,
            "averages");
    for (int k = 0; k < 9; ++k) REQUIRE(Pa[k] == Pb[k], "P_av differs");
    REQUIRE(dgx_commit_increment(dev_rve) == DGX_OK && dgx_commit_increment(host_rve) == DGX_OK, "commit");
    REQUIRE(cudaMemcpy(F0.data(), fp.F0, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost) == cudaSuccess, "read F0");
    for (int64_t k = 0; k < 9 * N; ++k) REQUIRE(F0[k] == F[k], "committed F0 differs from F");
  }
  // the host-copy path copied fields through host memory, the device path did not
  int64_t cd[10], ch[10];
  REQUIRE(dgx_counters(dev_rve, cd) == DGX_OK && dgx_counters(host_rve, ch) == DGX_OK, "counters");
  REQUIRE(cd[6] < 9 * N * 8 && cd[7] < 9 * N * 8, "device path copied fields through the host (%lld / %lld bytes)",
          (long long)cd[6], (long long)cd[7]);
  REQUIRE(ch[7] >= 2 * 90 * N * 8, "host path byte count");
  dgx_rve_destroy(dev_rve);
  dgx_rve_destroy(host_rve);
  std::printf("ok %d %d %d %lld\n", cells[0], cells[1], cells[2], (long long)N);
  return 0;
}
