// h5lite.hpp -- minimal HDF5 file writer and reader for result and restart files.
//
// No HDF5 library is available where the solver runs, so the files are written
// directly in the format of the public "HDF5 File Format Specification Version 2.0":
// superblock version 0 (8-byte offsets and lengths), version-1 object headers,
// old-style groups (symbol-table message, one-level v1 group B-tree, symbol-table
// nodes, local heap), contiguous datasets of IEEE float64 / int32 / fixed-length
// strings / a {label string, entry int64} compound, and version-1 attribute
// messages.  Raw data is appended while writing; all metadata (object headers,
// group structures, superblock) is written by close(), so a file is valid only
// after close().  The reader understands exactly these files (used for restarts).
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace h5lite {

constexpr uint64_t UNDEF = ~0ULL;
constexpr int LEAF_K = 16;        // symbol-table node: up to 32 entries
constexpr int INTERNAL_K = 64;    // group B-tree node: up to 128 symbol-table nodes

enum Kind { F64 = 0, I32 = 1, STR = 2, LABEL_ENTRY = 3, SPACE_STR = 4, I64 = 5 };

struct Attr {
  std::string name;
  Kind kind = F64;
  std::vector<uint64_t> dims;    // empty: scalar
  std::vector<double> f;
  std::vector<int32_t> i;
  std::string s;
};

struct Node {
  std::string name;
  bool group = true;
  std::vector<std::unique_ptr<Node>> kids;
  std::vector<Attr> attrs;
  // dataset
  Kind kind = F64;
  std::vector<uint64_t> dims;
  uint64_t data_addr = UNDEF, data_size = 0;
  uint32_t str_len = 0;          // STR length (with terminator) / LABEL_ENTRY label length
  // written by close()
  uint64_t header = 0, btree = 0, heap = 0;
  Node* child(const std::string& n) {
    for (auto& k : kids) if (k->name == n) return k.get();
    return nullptr;
  }
};

class Bytes {
 public:
  std::vector<uint8_t> b;
  void u8(uint8_t v) { b.push_back(v); }
  void u16(uint16_t v) { for (int k = 0; k < 2; ++k) b.push_back((uint8_t)(v >> (8 * k))); }
  void u32(uint32_t v) { for (int k = 0; k < 4; ++k) b.push_back((uint8_t)(v >> (8 * k))); }
  void u64(uint64_t v) { for (int k = 0; k < 8; ++k) b.push_back((uint8_t)(v >> (8 * k))); }
  void raw(const void* p, size_t n) { b.insert(b.end(), (const uint8_t*)p, (const uint8_t*)p + n); }
  void pad8() { while (b.size() % 8) b.push_back(0); }
  size_t size() const { return b.size(); }
};

inline void put_dtype(Bytes& o, Kind k, uint32_t str_len) {
  if (k == F64) {
    o.u8(0x11); o.u8(0x20); o.u8(63); o.u8(0); o.u32(8);            // IEEE float, LE, implied MSB, sign bit 63
    o.u16(0); o.u16(64); o.u8(52); o.u8(11); o.u8(0); o.u8(52); o.u32(1023);
  } else if (k == I32) {
    o.u8(0x10); o.u8(0x08); o.u8(0); o.u8(0); o.u32(4);             // fixed point, LE, signed
    o.u16(0); o.u16(32);
  } else if (k == STR) {
    o.u8(0x13); o.u8(0x00); o.u8(0); o.u8(0); o.u32(str_len);       // null-terminated ASCII
  } else if (k == SPACE_STR) {
    o.u8(0x13); o.u8(0x02); o.u8(0); o.u8(0); o.u32(str_len);       // space-padded ASCII, no terminator
  } else if (k == I64) {
    o.u8(0x10); o.u8(0x08); o.u8(0); o.u8(0); o.u32(8);             // fixed point, LE, signed
    o.u16(0); o.u16(64);
  } else {                                                           // {label: string, entry: int64}
    o.u8(0x16); o.u8(2); o.u8(0); o.u8(0); o.u32(str_len + 8);
    const char* names[2] = {"label", "entry"};
    const uint32_t offs[2] = {0, str_len};
    for (int m = 0; m < 2; ++m) {
      o.raw(names[m], strlen(names[m]) + 1); o.pad8();
      o.u32(offs[m]); o.u8(0); o.u8(0); o.u8(0); o.u8(0);          // offset, rank 0, reserved
      o.u32(0); o.u32(0); for (int d = 0; d < 4; ++d) o.u32(0);    // permutation, reserved, dims
      put_dtype(o, m == 0 ? SPACE_STR : I64, str_len);
    }
  }
}
inline void put_dspace(Bytes& o, const std::vector<uint64_t>& dims) {
  o.u8(1); o.u8((uint8_t)dims.size()); o.u8(0); o.u8(0); o.u32(0);
  for (uint64_t d : dims) o.u64(d);
}
inline void put_msg(Bytes& hdr, uint16_t type, const Bytes& m, int& nmsg) {
  Bytes d = m; d.pad8();
  hdr.u16(type); hdr.u16((uint16_t)d.size()); hdr.u8(0); hdr.u8(0); hdr.u8(0); hdr.u8(0);
  hdr.raw(d.b.data(), d.size());
  nmsg++;
}
inline void put_attr(Bytes& hdr, const Attr& a, int& nmsg) {
  Bytes dt, ds, data;
  uint32_t sl = 0;
  if (a.kind == STR) sl = (uint32_t)a.s.size() + 1;
  put_dtype(dt, a.kind, sl);
  put_dspace(ds, a.dims);
  if (a.kind == F64) data.raw(a.f.data(), a.f.size() * 8);
  else if (a.kind == I32) data.raw(a.i.data(), a.i.size() * 4);
  else data.raw(a.s.c_str(), a.s.size() + 1);
  Bytes m;
  m.u8(1); m.u8(0); m.u16((uint16_t)(a.name.size() + 1)); m.u16((uint16_t)dt.size()); m.u16((uint16_t)ds.size());
  m.raw(a.name.c_str(), a.name.size() + 1); m.pad8();
  m.raw(dt.b.data(), dt.size()); m.pad8();
  m.raw(ds.b.data(), ds.size()); m.pad8();
  m.raw(data.b.data(), data.size());
  put_msg(hdr, 0x000C, m, nmsg);
}

class Writer {
 public:
  ~Writer() { if (f_) fclose(f_); }
  bool open(const std::string& path) {
    f_ = fopen(path.c_str(), "wb");
    if (!f_) return false;
    std::vector<uint8_t> zero(96, 0);
    fwrite(zero.data(), 1, zero.size(), f_);
    eof_ = 96;
    return true;
  }
  Node* group(const std::string& path) {
    Node* n = &root_;
    size_t p = 0;
    while (p < path.size()) {
      size_t q = path.find('/', p);
      if (q == std::string::npos) q = path.size();
      std::string part = path.substr(p, q - p);
      p = q + 1;
      if (part.empty()) continue;
      Node* c = n->child(part);
      if (!c) {
        n->kids.emplace_back(new Node());
        c = n->kids.back().get();
        c->name = part;
      }
      n = c;
    }
    return n;
  }
  // raw data is appended now (8-byte aligned); the dataset's header comes at close()
  Node* dataset(const std::string& path, Kind kind, const std::vector<uint64_t>& dims, const void* data, size_t bytes,
                uint32_t str_len = 0) {
    size_t s = path.rfind('/');
    Node* g = group(s == std::string::npos ? "" : path.substr(0, s));
    g->kids.emplace_back(new Node());
    Node* d = g->kids.back().get();
    d->name = s == std::string::npos ? path : path.substr(s + 1);
    d->group = false; d->kind = kind; d->dims = dims; d->str_len = str_len;
    align();
    d->data_addr = eof_; d->data_size = bytes;
    if (bytes) fwrite(data, 1, bytes, f_);
    eof_ += bytes;
    return d;
  }
  Node* root() { return &root_; }
  bool close() {
    if (!f_) return false;
    write_node(&root_);
    // superblock v0
    Bytes sb;
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    sb.raw(sig, 8);
    sb.u8(0); sb.u8(0); sb.u8(0); sb.u8(0); sb.u8(0); sb.u8(8); sb.u8(8); sb.u8(0);
    sb.u16(LEAF_K); sb.u16(INTERNAL_K); sb.u32(0);
    sb.u64(0); sb.u64(UNDEF); sb.u64(eof_); sb.u64(UNDEF);
    sb.u64(0); sb.u64(root_.header); sb.u32(1); sb.u32(0); sb.u64(root_.btree); sb.u64(root_.heap);
    fseek(f_, 0, SEEK_SET);
    fwrite(sb.b.data(), 1, sb.size(), f_);
    bool ok = ferror(f_) == 0;
    ok = (fclose(f_) == 0) && ok;
    f_ = nullptr;
    return ok;
  }

 private:
  FILE* f_ = nullptr;
  uint64_t eof_ = 0;
  Node root_;
  void align() {
    static const uint8_t z[8] = {0};
    if (eof_ % 8) { size_t n = 8 - eof_ % 8; fwrite(z, 1, n, f_); eof_ += n; }
  }
  uint64_t append(const Bytes& b) {
    align();
    uint64_t at = eof_;
    fwrite(b.b.data(), 1, b.size(), f_);
    eof_ += b.size();
    return at;
  }
  uint64_t header(const Bytes& msgs, int nmsg) {
    Bytes h;
    h.u8(1); h.u8(0); h.u16((uint16_t)nmsg); h.u32(1); h.u32((uint32_t)msgs.size()); h.u32(0);
    h.raw(msgs.b.data(), msgs.size());
    return append(h);
  }
  void write_node(Node* n) {
    Bytes msgs;
    int nmsg = 0;
    if (!n->group) {
      Bytes ds, dt, fill, lay;
      put_dspace(ds, n->dims);
      put_dtype(dt, n->kind, n->str_len);
      fill.u8(2); fill.u8(2); fill.u8(2); fill.u8(0);               // fill value v2: late, if set, undefined
      lay.u8(3); lay.u8(1); lay.u64(n->data_addr); lay.u64(n->data_size);
      put_msg(msgs, 0x0001, ds, nmsg);
      put_msg(msgs, 0x0003, dt, nmsg);
      put_msg(msgs, 0x0005, fill, nmsg);
      put_msg(msgs, 0x0008, lay, nmsg);
      for (auto& a : n->attrs) put_attr(msgs, a, nmsg);
      n->header = header(msgs, nmsg);
      return;
    }
    for (auto& k : n->kids) write_node(k.get());
    std::vector<Node*> kids;
    for (auto& k : n->kids) kids.push_back(k.get());
    std::sort(kids.begin(), kids.end(), [](Node* a, Node* b) { return strcmp(a->name.c_str(), b->name.c_str()) < 0; });
    // local heap: "" then the names, each padded to 8 bytes
    Bytes seg;
    seg.u64(0);
    std::vector<uint64_t> off;
    for (Node* k : kids) { off.push_back(seg.size()); seg.raw(k->name.c_str(), k->name.size() + 1); seg.pad8(); }
    // one 16-byte free block at the end (next = 1: none), as the HDF5 library lays out heaps
    const uint64_t free_at = seg.size();
    seg.u64(1); seg.u64(16);
    Bytes hp;
    hp.raw("HEAP", 4); hp.u8(0); hp.u8(0); hp.u8(0); hp.u8(0);
    hp.u64(seg.size()); hp.u64(free_at);
    uint64_t seg_addr_pos = hp.size();
    hp.u64(0);
    hp.raw(seg.b.data(), seg.size());
    align();
    uint64_t heap_at = eof_;
    uint64_t seg_at = heap_at + 32;
    memcpy(&hp.b[seg_addr_pos], &seg_at, 8);
    append(hp);
    // symbol-table nodes of up to 2 LEAF_K sorted entries
    std::vector<uint64_t> snods, last_key;
    for (size_t s = 0; s < kids.size(); s += 2 * LEAF_K) {
      size_t e = std::min(kids.size(), s + 2 * LEAF_K);
      Bytes sn;
      sn.raw("SNOD", 4); sn.u8(1); sn.u8(0); sn.u16((uint16_t)(e - s));
      for (size_t k = 0; k < 2 * (size_t)LEAF_K; ++k) {
        if (s + k < e) {
          Node* c = kids[s + k];
          sn.u64(off[s + k]); sn.u64(c->header);
          if (c->group) { sn.u32(1); sn.u32(0); sn.u64(c->btree); sn.u64(c->heap); }
          else { sn.u32(0); sn.u32(0); sn.u64(0); sn.u64(0); }
        } else {
          for (int w = 0; w < 5; ++w) sn.u64(0);
        }
      }
      snods.push_back(append(sn));
      last_key.push_back(off[e - 1]);
    }
    // one-level group B-tree over the symbol-table nodes
    Bytes bt;
    bt.raw("TREE", 4); bt.u8(0); bt.u8(0); bt.u16((uint16_t)snods.size()); bt.u64(UNDEF); bt.u64(UNDEF);
    bt.u64(0);
    for (size_t c = 0; c < snods.size(); ++c) { bt.u64(snods[c]); bt.u64(last_key[c]); }
    for (size_t c = snods.size(); c < 2 * (size_t)INTERNAL_K; ++c) { bt.u64(0); bt.u64(0); }
    n->btree = append(bt);
    n->heap = heap_at;
    Bytes st;
    st.u64(n->btree); st.u64(n->heap);
    put_msg(msgs, 0x0011, st, nmsg);
    for (auto& a : n->attrs) put_attr(msgs, a, nmsg);
    n->header = header(msgs, nmsg);
  }
};

inline Attr attr_str(const std::string& name, const std::string& v) {
  Attr a; a.name = name; a.kind = STR; a.s = v; return a;
}
inline Attr attr_f64(const std::string& name, const std::vector<double>& v, bool scalar = false) {
  Attr a; a.name = name; a.kind = F64; a.f = v; if (!scalar) a.dims = {v.size()}; return a;
}
inline Attr attr_i32(const std::string& name, const std::vector<int32_t>& v, bool scalar = false) {
  Attr a; a.name = name; a.kind = I32; a.i = v; if (!scalar) a.dims = {v.size()}; return a;
}

// ---------------------------------------------------------------- reader
class Reader {
 public:
  bool open(const std::string& path) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (n < 96) { fclose(f); return false; }
    b_.resize((size_t)n);
    size_t got = fread(b_.data(), 1, b_.size(), f);
    fclose(f);
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    if (got != b_.size() || memcmp(b_.data(), sig, 8) != 0 || b_[8] != 0 || b_[13] != 8 || b_[14] != 8) return false;
    root_ = u64(24 + 32 + 8);
    return true;
  }
  // dataset data as raw bytes (contiguous layout); dims out
  bool read(const std::string& path, std::vector<uint8_t>& out, std::vector<uint64_t>* dims = nullptr) {
    uint64_t h = lookup(path);
    if (h == UNDEF) return false;
    uint64_t addr = UNDEF, size = 0;
    for (auto& m : messages(h)) {
      if (m.type == 0x0008 && b_[m.at] == 3 && b_[m.at + 1] == 1) { addr = u64(m.at + 2); size = u64(m.at + 10); }
      if (m.type == 0x0001 && dims) {
        dims->clear();
        for (int d = 0; d < b_[m.at + 1]; ++d) dims->push_back(u64(m.at + 8 + 8 * d));
      }
    }
    if (addr == UNDEF || addr + size > b_.size()) return false;
    out.assign(b_.begin() + addr, b_.begin() + addr + size);
    return true;
  }
  bool exists(const std::string& path) { return lookup(path) != UNDEF; }

 private:
  std::vector<uint8_t> b_;
  uint64_t root_ = 0;
  struct Msg { uint16_t type; uint64_t at; uint16_t size; };
  uint64_t u64(uint64_t p) const { uint64_t v; memcpy(&v, &b_[p], 8); return v; }
  uint16_t u16(uint64_t p) const { uint16_t v; memcpy(&v, &b_[p], 2); return v; }
  uint32_t u32(uint64_t p) const { uint32_t v; memcpy(&v, &b_[p], 4); return v; }
  std::vector<Msg> messages(uint64_t h) const {
    std::vector<Msg> out;
    if (h + 16 > b_.size() || b_[h] != 1) return out;
    int n = u16(h + 2);
    uint64_t p = h + 16, end = h + 16 + u32(h + 8);
    for (int k = 0; k < n && p + 8 <= end && end <= b_.size(); ++k) {
      Msg m{u16(p), p + 8, u16(p + 2)};
      out.push_back(m);
      p += 8 + m.size;
    }
    return out;
  }
  uint64_t lookup(const std::string& path) const {
    uint64_t h = root_;
    size_t p = 0;
    while (p < path.size()) {
      size_t q = path.find('/', p);
      if (q == std::string::npos) q = path.size();
      std::string part = path.substr(p, q - p);
      p = q + 1;
      if (part.empty()) continue;
      uint64_t bt = UNDEF, hp = UNDEF;
      for (auto& m : messages(h)) if (m.type == 0x0011) { bt = u64(m.at); hp = u64(m.at + 8); }
      if (bt == UNDEF || bt + 24 > b_.size()) return UNDEF;
      uint64_t seg = u64(hp + 24);
      int nc = u16(bt + 6);
      uint64_t found = UNDEF;
      for (int c = 0; c < nc && found == UNDEF; ++c) {
        uint64_t sn = u64(bt + 24 + 8 + 16 * c);
        int ns = u16(sn + 6);
        for (int e = 0; e < ns; ++e) {
          uint64_t ent = sn + 8 + 40 * e;
          const char* nm = (const char*)&b_[seg + u64(ent)];
          if (part == nm) { found = u64(ent + 8); break; }
        }
      }
      if (found == UNDEF) return UNDEF;
      h = found;
    }
    return h;
  }
};

}  // namespace h5lite
