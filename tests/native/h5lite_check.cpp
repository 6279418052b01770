// Writes an HDF5 file with the result writer (h5lite.hpp) -- nested groups, float64,
// int32, string and {label, entry} datasets, attributes, a group with more members than
// one symbol-table node holds -- then reads it back with the restart reader.
// Usage: h5lite_check <file>; prints "ok" and exits 0 when the read-back matches.
#include <cstdio>
#include <string>
#include <vector>

#include "../../solver_cpp_gb300/csrc/h5lite.hpp"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  {
    h5lite::Writer w;
    if (!w.open(argv[1])) return 3;
    w.root()->attrs.push_back(h5lite::attr_i32("DADF5_version_major", {1}, true));
    w.root()->attrs.push_back(h5lite::attr_str("creator", "check"));
    w.group("geometry")->attrs.push_back(h5lite::attr_i32("cells", {2, 3, 4}));
    std::vector<double> a(2 * 3 * 3);
    for (size_t k = 0; k < a.size(); ++k) a[k] = 0.5 * k - 1.0;
    h5lite::Node* d = w.dataset("increment_0/phase/alpha/mechanical/F", h5lite::F64, {2, 3, 3}, a.data(), a.size() * 8);
    d->attrs.push_back(h5lite::attr_str("unit", "1"));
    w.group("increment_0")->attrs.push_back(h5lite::attr_f64("t/s", {2.5}, true));
    std::vector<int32_t> iv = {7, -8, 9};
    w.dataset("solver/ints", h5lite::I32, {3}, iv.data(), 12);
    std::string txt = "line one\nline two";
    w.dataset("setup/load.yaml", h5lite::STR, {}, txt.c_str(), txt.size() + 1, (uint32_t)txt.size() + 1);
    std::vector<uint8_t> rec(3 * (5 + 8), 0);
    for (int e = 0; e < 3; ++e) { memcpy(&rec[e * 13], "alpha", 5); int64_t v = e; memcpy(&rec[e * 13 + 5], &v, 8); }
    w.dataset("cell_to/phase", h5lite::LABEL_ENTRY, {3, 1}, rec.data(), rec.size(), 5);
    for (int k = 0; k < 70; ++k) {              // more than one symbol-table node of entries
      double v = k;
      w.dataset("many/d" + std::to_string(k), h5lite::F64, {1}, &v, 8);
    }
    w.group("increment_0/homogenization/SX/mechanical");
    if (!w.close()) return 4;
  }
  h5lite::Reader r;
  if (!r.open(argv[1])) return 5;
  std::vector<uint8_t> b;
  std::vector<uint64_t> dims;
  if (!r.read("increment_0/phase/alpha/mechanical/F", b, &dims) || b.size() != 18 * 8 || dims.size() != 3) return 6;
  double v;
  memcpy(&v, &b[8 * 17], 8);
  if (v != 0.5 * 17 - 1.0) return 7;
  for (int k = 0; k < 70; ++k) {
    if (!r.read("many/d" + std::to_string(k), b) || b.size() != 8) return 8;
    memcpy(&v, b.data(), 8);
    if (v != k) return 9;
  }
  if (r.exists("many/d70") || !r.exists("increment_0/homogenization/SX/mechanical")) return 10;
  printf("ok\n");
  return 0;
}
