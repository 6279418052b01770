// vti.cpp -- VTK ImageData (.vti) geometry reader of the C ABI, from a file's content
// held in memory.
//
// Replaces f_VTI_readCellsSizeOrigin and f_VTI_readDataset_int (reference
// src/grid/discretization_grid.h:19-21, used by DiscretizationGrid::init,
// discretization_grid.cpp:8-20; the Fortran readers are src/VTI.f90):
//   cells  = WholeExtent upper - lower bounds per axis,
//   size   = cells x Spacing,
//   origin = Origin,
//   dataset = the cell-data array of the given name (DAMASK: "material"), x fastest.
// Supported encodings (what DAMASK and VTK write): format="ascii" and inline
// format="binary" (base64), raw or vtkZLibDataCompressor blocks, header_type UInt32 or
// UInt64, LittleEndian, any integer element type.  The zlib blocks are inflated by
// the decoder below (RFC 1950 / 1951), so the library needs no zlib.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dgx.h"

namespace dgx { void set_err(const char* fmt, ...); }

namespace {

using dgx::set_err;

// ------------------------------------------------------------------ XML scanning
// the text of the first start tag <name ...> at or after pos (without '<' name and '>')
bool find_tag(const std::string& s, const char* name, size_t from, size_t* attr_begin, size_t* attr_end,
              size_t* after) {
  const std::string open = std::string("<") + name;
  size_t p = from;
  for (;;) {
    p = s.find(open, p);
    if (p == std::string::npos) return false;
    const char c = p + open.size() < s.size() ? s[p + open.size()] : '\0';
    if (c == ' ' || c == '>' || c == '\t' || c == '\n' || c == '\r' || c == '/') break;
    p += open.size();
  }
  const size_t e = s.find('>', p);
  if (e == std::string::npos) return false;
  *attr_begin = p + open.size();
  *attr_end = e;
  *after = e + 1;
  return true;
}

bool attr(const std::string& s, size_t b, size_t e, const char* key, std::string* out) {
  const std::string k = key;
  size_t p = b;
  while (p < e) {
    p = s.find(k, p);
    if (p == std::string::npos || p >= e) return false;
    const bool start_ok = p == b || s[p - 1] == ' ' || s[p - 1] == '\t' || s[p - 1] == '\n' || s[p - 1] == '\r';
    size_t q = p + k.size();
    while (q < e && (s[q] == ' ' || s[q] == '\t')) ++q;
    if (start_ok && q < e && s[q] == '=') {
      ++q;
      while (q < e && (s[q] == ' ' || s[q] == '\t')) ++q;
      if (q < e && (s[q] == '"' || s[q] == '\'')) {
        const char quote = s[q];
        const size_t r = s.find(quote, q + 1);
        if (r == std::string::npos || r > e) return false;
        *out = s.substr(q + 1, r - q - 1);
        return true;
      }
    }
    p += k.size();
  }
  return false;
}

bool parse_numbers(const std::string& v, int want, double* out) {
  const char* c = v.c_str();
  for (int i = 0; i < want; ++i) {
    char* end = nullptr;
    out[i] = strtod(c, &end);
    if (end == c) return false;
    c = end;
  }
  return true;
}

// ------------------------------------------------------------------ base64
int b64v(char c) {
  if (c >= 'A' && c <= 'Z') return c - 'A';
  if (c >= 'a' && c <= 'z') return c - 'a' + 26;
  if (c >= '0' && c <= '9') return c - '0' + 52;
  if (c == '+') return 62;
  if (c == '/') return 63;
  return -1;
}

// decode base64 characters (whitespace ignored) up to the end or to a padded quantum
// ('='); *used receives the number of characters consumed (through the padding)
bool b64decode(const char* s, size_t n, std::vector<uint8_t>& out, size_t* used) {
  uint32_t acc = 0;
  int bits = 0, quantum = 0;
  size_t i = 0;
  for (; i < n; ++i) {
    const char c = s[i];
    if (c == ' ' || c == '\n' || c == '\r' || c == '\t') continue;
    if (c == '=') {
      // padding ends this encoded block: skip the rest of the padding
      while (i < n && (s[i] == '=' || s[i] == ' ' || s[i] == '\n' || s[i] == '\r' || s[i] == '\t')) ++i;
      *used = i;
      return true;
    }
    const int v = b64v(c);
    if (v < 0) return false;
    acc = (acc << 6) | (uint32_t)v;
    bits += 6;
    quantum = (quantum + 1) & 3;
    if (bits >= 8) {
      bits -= 8;
      out.push_back((uint8_t)((acc >> bits) & 0xff));
    }
  }
  (void)quantum;
  *used = i;
  return true;
}

// ------------------------------------------------------------------ inflate (RFC 1951)
struct BitReader {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t buf = 0;
  int cnt = 0;
  bool bad = false;
  int bits(int need) {
    uint32_t v = buf;
    while (cnt < need) {
      if (pos >= n) { bad = true; return 0; }
      v |= (uint32_t)p[pos++] << cnt;
      cnt += 8;
    }
    buf = v >> need;
    cnt -= need;
    return (int)(v & ((1u << need) - 1u));
  }
};

// canonical Huffman code: count[len] codes of each length, symbols in code order
struct Huffman {
  short count[16];
  short symbol[320];
};

bool build(Huffman& h, const short* length, int n) {
  for (int l = 0; l < 16; ++l) h.count[l] = 0;
  for (int s = 0; s < n; ++s) h.count[length[s]]++;
  if (h.count[0] == n) return true;            // no codes: only valid if never used
  int left = 1;
  for (int l = 1; l < 16; ++l) {
    left <<= 1;
    left -= h.count[l];
    if (left < 0) return false;                // over-subscribed
  }
  short offs[16];
  offs[1] = 0;
  for (int l = 1; l < 15; ++l) offs[l + 1] = (short)(offs[l] + h.count[l]);
  for (int s = 0; s < n; ++s)
    if (length[s] != 0) h.symbol[offs[length[s]]++] = (short)s;
  return true;
}

// decode one symbol, reading the code bit by bit (codes are stored MSB first)
int decode(BitReader& br, const Huffman& h) {
  int code = 0, first = 0, index = 0;
  for (int l = 1; l < 16; ++l) {
    code |= br.bits(1);
    if (br.bad) return -1;
    const int count = h.count[l];
    if (code - count < first) return h.symbol[index + (code - first)];
    index += count;
    first += count;
    first <<= 1;
    code <<= 1;
  }
  return -1;
}

const short LBASE[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115,
                         131, 163, 195, 227, 258};
const short LEXT[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const short DBASE[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537,
                         2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const short DEXT[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool codes(BitReader& br, std::vector<uint8_t>& out, const Huffman& lc, const Huffman& dc) {
  for (;;) {
    int sym = decode(br, lc);
    if (sym < 0) return false;
    if (sym < 256) { out.push_back((uint8_t)sym); continue; }
    if (sym == 256) return true;
    sym -= 257;
    if (sym >= 29) return false;
    const int len = LBASE[sym] + br.bits(LEXT[sym]);
    const int ds = decode(br, dc);
    if (ds < 0 || ds >= 30) return false;
    const size_t dist = (size_t)DBASE[ds] + (size_t)br.bits(DEXT[ds]);
    if (br.bad || dist > out.size()) return false;
    const size_t from = out.size() - dist;
    for (int k = 0; k < len; ++k) out.push_back(out[from + k]);
  }
}

bool inflate_raw(const uint8_t* p, size_t n, std::vector<uint8_t>& out) {
  BitReader br{p, n};
  int last;
  do {
    last = br.bits(1);
    const int type = br.bits(2);
    if (br.bad) return false;
    if (type == 0) {                            // stored
      br.buf = 0; br.cnt = 0;                   // to the byte boundary
      if (br.pos + 4 > n) return false;
      const unsigned len = p[br.pos] | (p[br.pos + 1] << 8);
      const unsigned nlen = p[br.pos + 2] | (p[br.pos + 3] << 8);
      br.pos += 4;
      if (len != (~nlen & 0xffffu) || br.pos + len > n) return false;
      out.insert(out.end(), p + br.pos, p + br.pos + len);
      br.pos += len;
    } else if (type == 1) {                     // fixed codes (tables built once, thread-safe)
      struct Fixed {
        Huffman lc, dc;
        Fixed() {
          short len[288];
          int s = 0;
          for (; s < 144; ++s) len[s] = 8;
          for (; s < 256; ++s) len[s] = 9;
          for (; s < 280; ++s) len[s] = 7;
          for (; s < 288; ++s) len[s] = 8;
          build(lc, len, 288);
          short dl[30];
          for (int d = 0; d < 30; ++d) dl[d] = 5;
          build(dc, dl, 30);
        }
      };
      static const Fixed fixed;
      if (!codes(br, out, fixed.lc, fixed.dc)) return false;
    } else if (type == 2) {                     // dynamic codes
      const int nlen = br.bits(5) + 257, ndist = br.bits(5) + 1, ncode = br.bits(4) + 4;
      if (br.bad || nlen > 286 || ndist > 30) return false;
      static const short ORDER[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      short lengths[320];
      for (int k = 0; k < 19; ++k) lengths[ORDER[k]] = k < ncode ? (short)br.bits(3) : 0;
      Huffman lencode, lc, dc;
      if (br.bad || !build(lencode, lengths, 19)) return false;
      int idx = 0;
      while (idx < nlen + ndist) {
        int sym = decode(br, lencode);
        if (sym < 0) return false;
        if (sym < 16) { lengths[idx++] = (short)sym; continue; }
        short v = 0;
        int rep;
        if (sym == 16) {
          if (idx == 0) return false;
          v = lengths[idx - 1];
          rep = 3 + br.bits(2);
        } else if (sym == 17) {
          rep = 3 + br.bits(3);
        } else {
          rep = 11 + br.bits(7);
        }
        if (br.bad || idx + rep > nlen + ndist) return false;
        while (rep--) lengths[idx++] = v;
      }
      if (lengths[256] == 0) return false;      // no end-of-block code
      if (!build(lc, lengths, nlen) || !build(dc, lengths + nlen, ndist)) return false;
      if (!codes(br, out, lc, dc)) return false;
    } else {
      return false;
    }
  } while (!last);
  return true;
}

// zlib stream (RFC 1950): header, deflate data, Adler-32 of the output
bool inflate_zlib(const uint8_t* p, size_t n, std::vector<uint8_t>& out) {
  if (n < 6) return false;
  const int cmf = p[0], flg = p[1];
  if ((cmf & 0x0f) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) return false;
  const size_t start = out.size();
  if (!inflate_raw(p + 2, n - 2, out)) return false;
  uint32_t a = 1, b = 0;
  for (size_t k = start; k < out.size(); ++k) { a = (a + out[k]) % 65521u; b = (b + a) % 65521u; }
  // the checksum follows the deflate data; its position is the end of the stream
  const uint32_t want = ((uint32_t)p[n - 4] << 24) | ((uint32_t)p[n - 3] << 16) | ((uint32_t)p[n - 2] << 8) | p[n - 1];
  return ((b << 16) | a) == want;
}

// ------------------------------------------------------------------ the document
struct Vti {
  int32_t cells[3];
  double size[3], origin[3];
  bool compressed = false;
  int header_bytes = 4;
  size_t celldata_b = 0, celldata_e = 0;        // content of <CellData> ... </CellData>
};

dgx_status parse_head(const std::string& s, Vti* v) {
  size_t ab, ae, after;
  if (!find_tag(s, "VTKFile", 0, &ab, &ae, &after)) { set_err("vti: no VTKFile element"); return DGX_ERR_ARG; }
  std::string t;
  if (!attr(s, ab, ae, "type", &t) || t != "ImageData") { set_err("vti: not an ImageData file"); return DGX_ERR_ARG; }
  if (attr(s, ab, ae, "byte_order", &t) && t != "LittleEndian") { set_err("vti: only LittleEndian data"); return DGX_ERR_UNSUPPORTED; }
  if (attr(s, ab, ae, "header_type", &t)) {
    if (t == "UInt64") v->header_bytes = 8;
    else if (t != "UInt32") { set_err("vti: header_type %s", t.c_str()); return DGX_ERR_UNSUPPORTED; }
  }
  if (attr(s, ab, ae, "compressor", &t)) {
    if (t != "vtkZLibDataCompressor") { set_err("vti: compressor %s", t.c_str()); return DGX_ERR_UNSUPPORTED; }
    v->compressed = true;
  }
  if (!find_tag(s, "ImageData", after, &ab, &ae, &after)) { set_err("vti: no ImageData element"); return DGX_ERR_ARG; }
  double ext[6], sp[3], org[3] = {0.0, 0.0, 0.0};
  if (!attr(s, ab, ae, "WholeExtent", &t) || !parse_numbers(t, 6, ext)) { set_err("vti: WholeExtent"); return DGX_ERR_ARG; }
  if (!attr(s, ab, ae, "Spacing", &t) || !parse_numbers(t, 3, sp)) { set_err("vti: Spacing"); return DGX_ERR_ARG; }
  if (attr(s, ab, ae, "Origin", &t) && !parse_numbers(t, 3, org)) { set_err("vti: Origin"); return DGX_ERR_ARG; }
  for (int i = 0; i < 3; ++i) {
    v->cells[i] = (int32_t)(ext[2 * i + 1] - ext[2 * i]);
    if (v->cells[i] < 1 || !(sp[i] > 0.0)) { set_err("vti: invalid cells or spacing"); return DGX_ERR_ARG; }
    v->size[i] = v->cells[i] * sp[i];
    v->origin[i] = org[i];
  }
  if (find_tag(s, "CellData", after, &ab, &ae, &after)) {
    const size_t e = s.find("</CellData>", after);
    if (e != std::string::npos) { v->celldata_b = after; v->celldata_e = e; }
  }
  return DGX_OK;
}

uint64_t le(const uint8_t* p, int bytes) {
  uint64_t v = 0;
  for (int k = bytes - 1; k >= 0; --k) v = (v << 8) | p[k];
  return v;
}

// decode one inline binary DataArray body into raw bytes
dgx_status decode_binary(const std::string& s, size_t b, size_t e, const Vti& v, std::vector<uint8_t>& raw) {
  const int hb = v.header_bytes;
  while (b < e && (s[b] == ' ' || s[b] == '\n' || s[b] == '\r' || s[b] == '\t')) ++b;
  const char* txt = s.data() + b;
  const size_t n = e - b;
  if (!v.compressed) {
    // header (byte count) and data, each base64-encoded on its own or as one stream
    std::vector<uint8_t> all;
    size_t used = 0;
    if (!b64decode(txt, n, all, &used)) { set_err("vti: bad base64"); return DGX_ERR_ARG; }
    if (used < n) {                             // the header block was padded: data follow
      size_t used2 = 0;
      std::vector<uint8_t> rest;
      if (!b64decode(txt + used, n - used, rest, &used2)) { set_err("vti: bad base64"); return DGX_ERR_ARG; }
      all.insert(all.end(), rest.begin(), rest.end());
    }
    if (all.size() < (size_t)hb) { set_err("vti: short data"); return DGX_ERR_ARG; }
    const uint64_t count = le(all.data(), hb);
    if (all.size() < hb + count) { set_err("vti: data shorter than its header"); return DGX_ERR_ARG; }
    raw.assign(all.begin() + hb, all.begin() + hb + count);
    return DGX_OK;
  }
  // compressed: header [nblocks, block size, last block size, compressed sizes...]
  // encoded on its own, then the concatenated zlib blocks
  std::vector<uint8_t> h0;
  size_t used = 0;
  const size_t first = ((size_t)hb + 2) / 3 * 4;
  if (n < first || !b64decode(txt, first, h0, &used) || h0.size() < (size_t)hb) { set_err("vti: bad header"); return DGX_ERR_ARG; }
  const uint64_t nb = le(h0.data(), hb);
  if (nb > (1u << 24)) { set_err("vti: block count"); return DGX_ERR_ARG; }
  const size_t hlen = (size_t)hb * (3 + nb);
  const size_t hchars = (hlen + 2) / 3 * 4;
  std::vector<uint8_t> hdr;
  if (n < hchars || !b64decode(txt, hchars, hdr, &used) || hdr.size() < hlen) { set_err("vti: bad header"); return DGX_ERR_ARG; }
  std::vector<uint8_t> data;
  size_t used2 = 0;
  if (!b64decode(txt + hchars, n - hchars, data, &used2)) { set_err("vti: bad base64"); return DGX_ERR_ARG; }
  size_t off = 0;
  for (uint64_t k = 0; k < nb; ++k) {
    const uint64_t cs = le(hdr.data() + hb * (3 + k), hb);
    if (off + cs > data.size()) { set_err("vti: compressed block beyond the data"); return DGX_ERR_ARG; }
    if (!inflate_zlib(data.data() + off, (size_t)cs, raw)) { set_err("vti: corrupt zlib block %llu", (unsigned long long)k); return DGX_ERR_ARG; }
    off += cs;
  }
  return DGX_OK;
}

struct IntType { const char* name; int bytes; bool is_signed; };
const IntType INT_TYPES[] = {{"Int8", 1, true},   {"UInt8", 1, false},  {"Int16", 2, true}, {"UInt16", 2, false},
                             {"Int32", 4, true},  {"UInt32", 4, false}, {"Int64", 8, true}, {"UInt64", 8, false}};

}  // namespace

extern "C" dgx_status dgx_vti_read_cells_size_origin(const char* content, int64_t length, int32_t cells[3],
                                                     double size[3], double origin[3]) {
  if (!content || length <= 0 || !cells || !size || !origin) { set_err("dgx_vti_read_cells_size_origin: null argument"); return DGX_ERR_ARG; }
  const std::string s(content, (size_t)length);
  Vti v;
  dgx_status st = parse_head(s, &v);
  if (st != DGX_OK) return st;
  for (int i = 0; i < 3; ++i) { cells[i] = v.cells[i]; size[i] = v.size[i]; origin[i] = v.origin[i]; }
  return DGX_OK;
}

extern "C" dgx_status dgx_vti_read_dataset_int(const char* content, int64_t length, const char* label,
                                               int32_t label_length, int32_t* dataset, int64_t* dataset_size) {
  if (!content || length <= 0 || !label || label_length <= 0 || !dataset_size) {
    set_err("dgx_vti_read_dataset_int: null argument"); return DGX_ERR_ARG;
  }
  const std::string s(content, (size_t)length);
  const std::string name(label, (size_t)label_length);
  Vti v;
  dgx_status st = parse_head(s, &v);
  if (st != DGX_OK) return st;
  if (v.celldata_e <= v.celldata_b) { set_err("vti: no CellData"); return DGX_ERR_ARG; }
  const int64_t ncell = (int64_t)v.cells[0] * v.cells[1] * v.cells[2];
  size_t pos = v.celldata_b, ab, ae, after;
  while (pos < v.celldata_e && find_tag(s, "DataArray", pos, &ab, &ae, &after) && ab < v.celldata_e) {
    const size_t close = s.find("</DataArray>", after);
    if (close == std::string::npos || close > v.celldata_e) break;
    pos = close + 12;
    std::string nm, type, fmt = "ascii";
    if (!attr(s, ab, ae, "Name", &nm) || nm != name) continue;
    if (!attr(s, ab, ae, "type", &type)) { set_err("vti: DataArray without type"); return DGX_ERR_ARG; }
    attr(s, ab, ae, "format", &fmt);
    const IntType* it = nullptr;
    for (const IntType& t : INT_TYPES)
      if (type == t.name) it = &t;
    if (!it) { set_err("vti: %s is not an integer array (%s)", name.c_str(), type.c_str()); return DGX_ERR_UNSUPPORTED; }
    if (*dataset_size < ncell || !dataset) {
      *dataset_size = ncell;
      set_err("vti: %s needs room for %lld values", name.c_str(), (long long)ncell);
      return DGX_ERR_ARG;
    }
    int64_t count = 0;
    if (fmt == "ascii") {
      const char* c = s.data() + after;
      const char* end = s.data() + close;
      while (c < end) {
        while (c < end && (*c == ' ' || *c == '\n' || *c == '\r' || *c == '\t')) ++c;
        if (c >= end) break;
        char* stop = nullptr;
        const long long x = strtoll(c, &stop, 10);
        if (stop == c) { set_err("vti: bad ascii value"); return DGX_ERR_ARG; }
        if (count >= ncell) { set_err("vti: %s has more values than cells", name.c_str()); return DGX_ERR_ARG; }
        if (x < INT32_MIN || x > INT32_MAX) { set_err("vti: value out of int32 range"); return DGX_ERR_ARG; }
        dataset[count++] = (int32_t)x;
        c = stop;
      }
    } else if (fmt == "binary") {
      std::vector<uint8_t> raw;
      st = decode_binary(s, after, close, v, raw);
      if (st != DGX_OK) return st;
      if (raw.size() % it->bytes) { set_err("vti: data size not a multiple of the element size"); return DGX_ERR_ARG; }
      count = (int64_t)(raw.size() / it->bytes);
      if (count != ncell) { set_err("vti: %s has %lld values for %lld cells", name.c_str(), (long long)count, (long long)ncell); return DGX_ERR_ARG; }
      for (int64_t k = 0; k < count; ++k) {
        const uint64_t u = le(raw.data() + k * it->bytes, it->bytes);
        int64_t x;
        if (it->is_signed) {
          const int sh = 64 - 8 * it->bytes;
          x = sh ? (int64_t)(u << sh) >> sh : (int64_t)u;
        } else {
          if (it->bytes == 8 && u > (uint64_t)INT64_MAX) { set_err("vti: value out of int32 range"); return DGX_ERR_ARG; }
          x = (int64_t)u;
        }
        if (x < INT32_MIN || x > INT32_MAX) { set_err("vti: value out of int32 range"); return DGX_ERR_ARG; }
        dataset[k] = (int32_t)x;
      }
    } else {
      set_err("vti: DataArray format %s", fmt.c_str());
      return DGX_ERR_UNSUPPORTED;
    }
    if (count != ncell) { set_err("vti: %s has %lld values for %lld cells", name.c_str(), (long long)count, (long long)ncell); return DGX_ERR_ARG; }
    *dataset_size = count;
    return DGX_OK;
  }
  set_err("vti: no cell data array named %s", name.c_str());
  return DGX_ERR_ARG;
}
