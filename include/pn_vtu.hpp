// pn_vtu.hpp -- a header-only reader and writer for the VTK XML files PanNDE's
// jobs and outputs use, written from the published VTK XML file-format
// description (no VTK library):
//   .vtu   <VTKFile type="UnstructuredGrid">: Points, Cells (connectivity,
//          offsets, types), PointData, CellData, FieldData
//   .pvtu  <VTKFile type="PUnstructuredGrid">: the pieces' array layout and
//          their file names
//   .vtt   <VTKFile type="Table">: RowData columns, FieldData
// Reading accepts DataArrays in ascii, inline binary (base64) and appended
// (raw or base64) form, UInt32 or UInt64 block headers, uncompressed or
// vtkZLibDataCompressor blocks (when <zlib.h> is available), little-endian.
// Writing produces inline base64 binary, UInt64 headers, uncompressed.
// Every numeric array is held as double (integer ids up to 2^53 are exact).
#pragma once
#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#if defined(__has_include)
#if __has_include(<zlib.h>)
#include <zlib.h>
#define PN_VTU_HAVE_ZLIB 1
#endif
#endif

namespace pnvtu {

struct DataArray {
  std::string name;
  std::string type = "Float64";  // VTK type name: Float32/64, Int8..Int64, UInt8..UInt64
  int components = 1;
  std::vector<double> values;      // tuples x components
  int64_t tuples() const { return components > 0 ? (int64_t)values.size() / components : 0; }
};

struct Grid {
  std::vector<double> points;         // [n_points][3]
  std::vector<double> connectivity;   // cell point ids
  std::vector<double> offsets;        // end of each cell in connectivity
  std::vector<double> types;          // VTK cell types (12 = hexahedron)
  std::vector<DataArray> point_data, cell_data, field_data;
  int64_t n_points() const { return (int64_t)points.size() / 3; }
  int64_t n_cells() const { return (int64_t)offsets.size(); }
  static const DataArray *find(const std::vector<DataArray> &v, const std::string &name) {
    for (auto &a : v)
      if (a.name == name) return &a;
    return nullptr;
  }
};

struct Table {
  std::vector<DataArray> columns;     // RowData
  std::vector<DataArray> field_data;
};

// ---- base64 (RFC 4648) ----------------------------------------------------
inline std::string b64_encode(const unsigned char *p, size_t n) {
  static const char *tab = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
  std::string out;
  out.reserve((n + 2) / 3 * 4);
  for (size_t i = 0; i < n; i += 3) {
    const uint32_t a = p[i], b = i + 1 < n ? p[i + 1] : 0, c = i + 2 < n ? p[i + 2] : 0;
    const uint32_t v = (a << 16) | (b << 8) | c;
    out += tab[(v >> 18) & 63];
    out += tab[(v >> 12) & 63];
    out += i + 1 < n ? tab[(v >> 6) & 63] : '=';
    out += i + 2 < n ? tab[v & 63] : '=';
  }
  return out;
}

// Decodes one base64 unit (the encoding of n bytes: 4*ceil(n/3) characters,
// the last quad padded with '='), starting at s[pos] and skipping white
// space; advances pos past the unit.
inline std::vector<unsigned char> b64_unit(const std::string &s, size_t &pos, size_t n) {
  auto val = [](char ch) -> int {
    if (ch >= 'A' && ch <= 'Z') return ch - 'A';
    if (ch >= 'a' && ch <= 'z') return ch - 'a' + 26;
    if (ch >= '0' && ch <= '9') return ch - '0' + 52;
    if (ch == '+') return 62;
    if (ch == '/') return 63;
    if (ch == '=') return 64;
    return -1;
  };
  const size_t nchars = (n + 2) / 3 * 4;
  std::vector<unsigned char> out;
  out.reserve(n);
  uint32_t quad[4];
  size_t got = 0, q = 0;
  while (got < nchars) {
    if (pos >= s.size()) throw std::runtime_error("vtu: base64 data ends early");
    const int v = val(s[pos++]);
    if (v < 0) continue;  // white space
    quad[q++] = (uint32_t)(v == 64 ? 0 : v);
    got++;
    if (q == 4) {
      const uint32_t w = (quad[0] << 18) | (quad[1] << 12) | (quad[2] << 6) | quad[3];
      const unsigned char b[3] = {(unsigned char)(w >> 16), (unsigned char)(w >> 8), (unsigned char)w};
      for (int k = 0; k < 3 && out.size() < n; k++) out.push_back(b[k]);
      q = 0;
    }
  }
  return out;
}

// the non-white-space character that closes a base64 unit of n bytes
inline char b64_unit_last(const std::string &s, size_t pos, size_t n) {
  const size_t nchars = (n + 2) / 3 * 4;
  size_t got = 0;
  char last = 0;
  while (got < nchars && pos < s.size()) {
    const char ch = s[pos++];
    if (ch == ' ' || ch == '\n' || ch == '\r' || ch == '\t') continue;
    last = ch;
    got++;
  }
  return last;
}

// ---- element types ---------------------------------------------------------
inline int type_size(const std::string &t) {
  if (t == "Float64" || t == "Int64" || t == "UInt64") return 8;
  if (t == "Float32" || t == "Int32" || t == "UInt32") return 4;
  if (t == "Int16" || t == "UInt16") return 2;
  if (t == "Int8" || t == "UInt8") return 1;
  throw std::runtime_error("vtu: unsupported data type " + t);
}

inline double load_value(const unsigned char *p, const std::string &t) {
  if (t == "Float64") { double v; std::memcpy(&v, p, 8); return v; }
  if (t == "Float32") { float v; std::memcpy(&v, p, 4); return v; }
  if (t == "Int64") { int64_t v; std::memcpy(&v, p, 8); return (double)v; }
  if (t == "UInt64") { uint64_t v; std::memcpy(&v, p, 8); return (double)v; }
  if (t == "Int32") { int32_t v; std::memcpy(&v, p, 4); return v; }
  if (t == "UInt32") { uint32_t v; std::memcpy(&v, p, 4); return v; }
  if (t == "Int16") { int16_t v; std::memcpy(&v, p, 2); return v; }
  if (t == "UInt16") { uint16_t v; std::memcpy(&v, p, 2); return v; }
  if (t == "Int8") return (double)(int8_t)p[0];
  return (double)p[0];  // UInt8
}

inline void store_value(unsigned char *p, const std::string &t, double v) {
  if (t == "Float64") { std::memcpy(p, &v, 8); return; }
  if (t == "Float32") { const float f = (float)v; std::memcpy(p, &f, 4); return; }
  if (t == "Int64") { const int64_t q = (int64_t)v; std::memcpy(p, &q, 8); return; }
  if (t == "UInt64") { const uint64_t q = (uint64_t)v; std::memcpy(p, &q, 8); return; }
  if (t == "Int32") { const int32_t q = (int32_t)v; std::memcpy(p, &q, 4); return; }
  if (t == "UInt32") { const uint32_t q = (uint32_t)v; std::memcpy(p, &q, 4); return; }
  if (t == "Int16") { const int16_t q = (int16_t)v; std::memcpy(p, &q, 2); return; }
  if (t == "UInt16") { const uint16_t q = (uint16_t)v; std::memcpy(p, &q, 2); return; }
  if (t == "Int8") { p[0] = (unsigned char)(int8_t)v; return; }
  p[0] = (unsigned char)v;
}

// ---- minimal XML scanning ----------------------------------------------------
struct Tag {
  std::string name;
  std::map<std::string, std::string> attr;
  bool closing = false, self_closing = false;
  size_t begin = 0, end = 0;  // [begin, end) of the tag text
};

// next tag at or after pos (comments and declarations skipped)
inline bool next_tag(const std::string &s, size_t &pos, Tag &t) {
  for (;;) {
    const size_t lt = s.find('<', pos);
    if (lt == std::string::npos) return false;
    if (s.compare(lt, 4, "<!--") == 0) {
      const size_t e = s.find("-->", lt);
      pos = e == std::string::npos ? s.size() : e + 3;
      continue;
    }
    if (s.compare(lt, 2, "<?") == 0 || s.compare(lt, 2, "<!") == 0) {
      const size_t e = s.find('>', lt);
      pos = e == std::string::npos ? s.size() : e + 1;
      continue;
    }
    const size_t gt = s.find('>', lt);
    if (gt == std::string::npos) return false;
    t = Tag();
    t.begin = lt;
    t.end = gt + 1;
    size_t i = lt + 1;
    if (s[i] == '/') { t.closing = true; i++; }
    size_t j = i;
    while (j < gt && !isspace((unsigned char)s[j]) && s[j] != '/') j++;
    t.name = s.substr(i, j - i);
    t.self_closing = s[gt - 1] == '/';
    // attributes name="value"
    size_t k = j;
    while (k < gt) {
      while (k < gt && (isspace((unsigned char)s[k]) || s[k] == '/')) k++;
      const size_t eq = s.find('=', k);
      if (eq == std::string::npos || eq > gt) break;
      std::string key = s.substr(k, eq - k);
      while (!key.empty() && isspace((unsigned char)key.back())) key.pop_back();
      const size_t q1 = s.find_first_of("\"'", eq);
      if (q1 == std::string::npos || q1 > gt) break;
      const size_t q2 = s.find(s[q1], q1 + 1);
      if (q2 == std::string::npos) break;
      t.attr[key] = s.substr(q1 + 1, q2 - q1 - 1);
      k = q2 + 1;
    }
    pos = gt + 1;
    return true;
  }
}

inline std::string attr_or(const Tag &t, const std::string &k, const std::string &d) {
  auto it = t.attr.find(k);
  return it == t.attr.end() ? d : it->second;
}

struct FileInfo {
  std::string header_type = "UInt32";
  bool zlib = false;
  std::string appended_encoding;
  size_t appended_start = std::string::npos;  // first byte after '_'
};

inline uint64_t read_uint(const unsigned char *p, int size) {
  if (size == 8) { uint64_t v; std::memcpy(&v, p, 8); return v; }
  uint32_t v;
  std::memcpy(&v, p, 4);
  return v;
}

// Decode one binary block (header + data) at s[pos]: raw bytes (appended
// raw) or base64 (inline, or appended base64).  In base64, an uncompressed
// block is either one unit (header and data together) or two (the header,
// then the data) -- a header of 4 or 8 bytes encoded on its own always ends
// in '=' padding, which tells the two apart; a compressed block is its
// header unit followed by one unit of all compressed bytes.
inline std::vector<unsigned char> read_block(const std::string &s, size_t pos, bool base64, const FileInfo &fi) {
  const size_t hs = fi.header_type == "UInt64" ? 8 : 4;
  auto raw = [&](size_t n) -> std::vector<unsigned char> {
    if (pos + n > s.size()) throw std::runtime_error("vtu: appended data ends early");
    std::vector<unsigned char> v(s.begin() + pos, s.begin() + pos + n);
    pos += n;
    return v;
  };
  if (!fi.zlib) {
    if (!base64) {
      const std::vector<unsigned char> h = raw(hs);
      return raw((size_t)read_uint(h.data(), (int)hs));
    }
    size_t p = pos;
    const std::vector<unsigned char> h = b64_unit(s, p, hs);  // leading bytes either way
    const size_t nbytes = (size_t)read_uint(h.data(), (int)hs);
    if (b64_unit_last(s, pos, hs) == '=') {  // separate units
      size_t p2 = pos;
      (void)b64_unit(s, p2, hs);
      return b64_unit(s, p2, nbytes);
    }
    size_t p3 = pos;
    std::vector<unsigned char> all = b64_unit(s, p3, hs + nbytes);
    return std::vector<unsigned char>(all.begin() + hs, all.end());
  }
#ifdef PN_VTU_HAVE_ZLIB
  // header [nblocks][block size][last block size][compressed sizes...]
  std::vector<unsigned char> h0;
  if (base64) {
    size_t p = pos;
    h0 = b64_unit(s, p, 3 * hs);
  } else {
    size_t p = pos;
    if (p + 3 * hs > s.size()) throw std::runtime_error("vtu: truncated compressed header");
    h0.assign(s.begin() + p, s.begin() + p + 3 * hs);
  }
  const uint64_t nb = read_uint(h0.data(), (int)hs), bsz = read_uint(h0.data() + hs, (int)hs),
                 last = read_uint(h0.data() + 2 * hs, (int)hs);
  const size_t hbytes = (size_t)(hs * (3 + nb));
  std::vector<unsigned char> hdr = base64 ? b64_unit(s, pos, hbytes) : raw(hbytes);
  uint64_t total = 0;
  for (uint64_t b = 0; b < nb; b++) total += read_uint(hdr.data() + hs * (3 + b), (int)hs);
  std::vector<unsigned char> comp = base64 ? b64_unit(s, pos, (size_t)total) : raw((size_t)total);
  std::vector<unsigned char> out;
  size_t at_c = 0;
  for (uint64_t b = 0; b < nb; b++) {
    const uint64_t csz = read_uint(hdr.data() + hs * (3 + b), (int)hs);
    uLongf usz = (uLongf)((b + 1 == nb && last != 0) ? last : bsz);
    const size_t at = out.size();
    out.resize(at + usz);
    if (uncompress(out.data() + at, &usz, comp.data() + at_c, (uLong)csz) != Z_OK)
      throw std::runtime_error("vtu: zlib block does not inflate");
    out.resize(at + usz);
    at_c += (size_t)csz;
  }
  return out;
#else
  (void)raw;
  throw std::runtime_error("vtu: compressed arrays need zlib, which this build lacks");
#endif
}

// DataArray whose start tag is t (content follows t.end)
inline DataArray read_array(const std::string &s, const Tag &t, const FileInfo &fi, size_t tuples_hint = 0) {
  DataArray a;
  a.name = attr_or(t, "Name", "");
  a.type = attr_or(t, "type", "Float64");
  a.components = std::stoi(attr_or(t, "NumberOfComponents", "1"));
  const std::string fmt = attr_or(t, "format", "ascii");
  const int es = type_size(a.type);
  if (fmt == "ascii") {
    if (t.self_closing) return a;
    const size_t e = s.find('<', t.end);
    std::istringstream in(s.substr(t.end, e - t.end));
    double v;
    while (in >> v) a.values.push_back(v);
    return a;
  }
  std::vector<unsigned char> bytes;
  if (fmt == "binary") {
    bytes = read_block(s, t.end, true, fi);
  } else if (fmt == "appended") {
    if (fi.appended_start == std::string::npos) throw std::runtime_error("vtu: no AppendedData section");
    const size_t off = (size_t)std::stoull(attr_or(t, "offset", "0"));
    bytes = read_block(s, fi.appended_start + off, fi.appended_encoding == "base64", fi);
  } else {
    throw std::runtime_error("vtu: unknown DataArray format " + fmt);
  }
  const size_t n = bytes.size() / (size_t)es;
  a.values.resize(n);
  for (size_t i = 0; i < n; i++) a.values[i] = load_value(bytes.data() + i * es, a.type);
  (void)tuples_hint;
  return a;
}

inline std::string slurp(const std::string &path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("vtu: cannot open " + path);
  std::ostringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

inline FileInfo file_info(const std::string &s) {
  FileInfo fi;
  size_t pos = 0;
  Tag t;
  while (next_tag(s, pos, t)) {
    if (t.name == "VTKFile" && !t.closing) {
      fi.header_type = attr_or(t, "header_type", "UInt32");
      fi.zlib = attr_or(t, "compressor", "").find("ZLib") != std::string::npos;
      if (attr_or(t, "byte_order", "LittleEndian") != "LittleEndian")
        throw std::runtime_error("vtu: big-endian files are not supported");
    }
    if (t.name == "AppendedData" && !t.closing) {
      fi.appended_encoding = attr_or(t, "encoding", "raw");
      const size_t us = s.find('_', t.end);
      fi.appended_start = us == std::string::npos ? std::string::npos : us + 1;
      break;  // raw bytes follow: stop scanning tags
    }
  }
  return fi;
}

// walk the DataArrays of the file (up to an AppendedData section), calling
// f(section, array) with section the enclosing Points / Cells / PointData /
// CellData / FieldData / RowData element name
template <typename F>
inline void each_array(const std::string &s, const FileInfo &fi, F &&f) {
  size_t pos = 0;
  Tag t;
  std::vector<std::string> stack;
  while (next_tag(s, pos, t)) {
    if (t.name == "AppendedData") break;
    if (t.name == "DataArray" || t.name == "Array") {
      if (t.closing) continue;
      DataArray a = read_array(s, t, fi);
      f(stack.empty() ? std::string() : stack.back(), a);
      if (!t.self_closing) {  // skip to its end tag
        const size_t e = s.find("</", t.end);
        if (e != std::string::npos) pos = s.find('>', e) + 1;
      }
      continue;
    }
    if (t.self_closing) continue;
    if (t.closing) {
      if (!stack.empty()) stack.pop_back();
    } else {
      stack.push_back(t.name);
    }
  }
}

inline Grid read_vtu(const std::string &path) {
  const std::string s = slurp(path);
  const FileInfo fi = file_info(s);
  Grid g;
  each_array(s, fi, [&](const std::string &sec, DataArray &a) {
    if (sec == "Points") g.points = std::move(a.values);
    else if (sec == "Cells") {
      if (a.name == "connectivity") g.connectivity = std::move(a.values);
      else if (a.name == "offsets") g.offsets = std::move(a.values);
      else if (a.name == "types") g.types = std::move(a.values);
    } else if (sec == "PointData") g.point_data.push_back(std::move(a));
    else if (sec == "CellData") g.cell_data.push_back(std::move(a));
    else if (sec == "FieldData") g.field_data.push_back(std::move(a));
  });
  if (g.points.size() % 3 != 0) throw std::runtime_error("vtu: points are not 3-D");
  return g;
}

inline Table read_vtt(const std::string &path) {
  const std::string s = slurp(path);
  const FileInfo fi = file_info(s);
  Table tb;
  each_array(s, fi, [&](const std::string &sec, DataArray &a) {
    if (sec == "RowData") tb.columns.push_back(std::move(a));
    else if (sec == "FieldData") tb.field_data.push_back(std::move(a));
  });
  return tb;
}

// ---- writing -------------------------------------------------------------
inline void write_array(std::ostream &o, const DataArray &a, const char *indent, bool field = false) {
  const int es = type_size(a.type);
  std::vector<unsigned char> blk(8 + a.values.size() * (size_t)es);
  const uint64_t nbytes = (uint64_t)a.values.size() * (uint64_t)es;
  std::memcpy(blk.data(), &nbytes, 8);
  for (size_t i = 0; i < a.values.size(); i++) store_value(blk.data() + 8 + i * es, a.type, a.values[i]);
  o << indent << "<DataArray type=\"" << a.type << "\"";
  if (!a.name.empty()) o << " Name=\"" << a.name << "\"";
  if (a.components != 1) o << " NumberOfComponents=\"" << a.components << "\"";
  if (field) o << " NumberOfTuples=\"" << a.tuples() << "\"";
  o << " format=\"binary\">\n" << indent << "  " << b64_encode(blk.data(), blk.size()) << "\n"
    << indent << "</DataArray>\n";
}

inline void write_field_data(std::ostream &o, const std::vector<DataArray> &fd) {
  if (fd.empty()) return;
  o << "    <FieldData>\n";
  for (auto &a : fd) write_array(o, a, "      ", true);
  o << "    </FieldData>\n";
}

inline void write_vtu(const std::string &path, const Grid &g) {
  std::ofstream o(path, std::ios::binary);
  if (!o) throw std::runtime_error("vtu: cannot write " + path);
  o << "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" "
       "byte_order=\"LittleEndian\" header_type=\"UInt64\">\n  <UnstructuredGrid>\n";
  write_field_data(o, g.field_data);
  o << "    <Piece NumberOfPoints=\"" << g.n_points() << "\" NumberOfCells=\"" << g.n_cells() << "\">\n";
  o << "      <PointData>\n";
  for (auto &a : g.point_data) write_array(o, a, "        ");
  o << "      </PointData>\n      <CellData>\n";
  for (auto &a : g.cell_data) write_array(o, a, "        ");
  o << "      </CellData>\n      <Points>\n";
  DataArray pts{"Points", "Float64", 3, g.points};
  write_array(o, pts, "        ");
  o << "      </Points>\n      <Cells>\n";
  write_array(o, DataArray{"connectivity", "Int64", 1, g.connectivity}, "        ");
  write_array(o, DataArray{"offsets", "Int64", 1, g.offsets}, "        ");
  write_array(o, DataArray{"types", "UInt8", 1, g.types}, "        ");
  o << "      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n";
}

// one-piece parallel header next to its piece file (file names relative)
inline void write_pvtu(const std::string &path, const Grid &g, const std::vector<std::string> &pieces) {
  std::ofstream o(path, std::ios::binary);
  if (!o) throw std::runtime_error("vtu: cannot write " + path);
  o << "<?xml version=\"1.0\"?>\n<VTKFile type=\"PUnstructuredGrid\" version=\"1.0\" "
       "byte_order=\"LittleEndian\" header_type=\"UInt64\">\n  <PUnstructuredGrid GhostLevel=\"0\">\n";
  o << "    <PPointData>\n";
  for (auto &a : g.point_data)
    o << "      <PDataArray type=\"" << a.type << "\" Name=\"" << a.name << "\"/>\n";
  o << "    </PPointData>\n    <PCellData>\n";
  for (auto &a : g.cell_data)
    o << "      <PDataArray type=\"" << a.type << "\" Name=\"" << a.name << "\"/>\n";
  o << "    </PCellData>\n    <PPoints>\n      <PDataArray type=\"Float64\" NumberOfComponents=\"3\"/>\n"
       "    </PPoints>\n";
  for (auto &p : pieces) o << "    <Piece Source=\"" << p << "\"/>\n";
  o << "  </PUnstructuredGrid>\n</VTKFile>\n";
}

inline void write_vtt(const std::string &path, const Table &t) {
  std::ofstream o(path, std::ios::binary);
  if (!o) throw std::runtime_error("vtu: cannot write " + path);
  int64_t rows = 0;
  for (auto &c : t.columns) rows = std::max<int64_t>(rows, c.tuples());
  o << "<?xml version=\"1.0\"?>\n<VTKFile type=\"Table\" version=\"1.0\" byte_order=\"LittleEndian\" "
       "header_type=\"UInt64\">\n  <Table>\n";
  write_field_data(o, t.field_data);
  o << "    <Piece NumberOfCols=\"" << t.columns.size() << "\" NumberOfRows=\"" << rows << "\">\n"
       "      <RowData>\n";
  for (auto &c : t.columns) write_array(o, c, "        ");
  o << "      </RowData>\n    </Piece>\n  </Table>\n</VTKFile>\n";
}

}  // namespace pnvtu
