// cdf_io.cpp -- netCDF classic (CDF-1/CDF-2) and CDL reading and writing
// for the column files of the reference's Cl_run_cdf / Cl_run_cdl drivers.
// The binary layout is the published netCDF classic format (header of
// dimensions, attributes and variables with big-endian values; data of each
// non-record variable contiguous at its offset, record variables interleaved
// by record).
#include "cdf_io.h"

#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

namespace socgpu {

int NcFile::dim_index(const std::string &n) const {
  for (size_t i = 0; i < dims.size(); ++i)
    if (dims[i].first == n) return (int)i;
  return -1;
}

const NcVar *NcFile::var(const std::string &n) const {
  for (const NcVar &v : vars)
    if (v.name == n) return &v;
  return nullptr;
}

size_t NcFile::dim_len(const std::string &n) const {
  int i = dim_index(n);
  return i < 0 ? 0 : dims[i].second;
}

namespace {

bool slurp(const std::string &path, std::string &out) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return false;
  std::ostringstream ss;
  ss << in.rdbuf();
  out = ss.str();
  return true;
}

// ---------------------------------------------------------------- binary
struct Reader {
  const std::string &b;
  size_t pos = 0;
  bool ok = true;
  explicit Reader(const std::string &buf) : b(buf) {}
  uint32_t u32() {
    if (pos + 4 > b.size()) { ok = false; return 0; }
    uint32_t v = ((uint32_t)(unsigned char)b[pos] << 24) | ((uint32_t)(unsigned char)b[pos + 1] << 16) |
                 ((uint32_t)(unsigned char)b[pos + 2] << 8) | (uint32_t)(unsigned char)b[pos + 3];
    pos += 4;
    return v;
  }
  uint64_t u64() {
    uint64_t hi = u32();
    return (hi << 32) | u32();
  }
  std::string name() {
    uint32_t n = u32();
    if (!ok || pos + n > b.size()) { ok = false; return ""; }
    std::string s = b.substr(pos, n);
    pos += (n + 3) & ~3u;
    return s;
  }
};

size_t type_size(int t) {
  switch (t) {
    case 1: case 2: return 1;
    case 3: return 2;
    case 4: case 5: return 4;
    case 6: return 8;
    default: return 0;
  }
}

double get_value(const std::string &b, size_t at, int t) {
  const unsigned char *p = (const unsigned char *)b.data() + at;
  switch (t) {
    case 1: return (double)(int8_t)p[0];
    case 2: return (double)p[0];
    case 3: return (double)(int16_t)(uint16_t)((p[0] << 8) | p[1]);
    case 4: return (double)(int32_t)(((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]);
    case 5: {
      uint32_t u = ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
      float f;
      std::memcpy(&f, &u, 4);
      return (double)f;
    }
    case 6: {
      uint64_t u = 0;
      for (int i = 0; i < 8; ++i) u = (u << 8) | p[i];
      double d;
      std::memcpy(&d, &u, 8);
      return d;
    }
    default: return 0.0;
  }
}

// Attribute list; text attributes are kept, others skipped.
bool read_atts(Reader &r, std::vector<std::pair<std::string, std::string>> *keep) {
  uint32_t tag = r.u32(), n = r.u32();
  if (!r.ok) return false;
  if (tag == 0 && n == 0) return true;
  if (tag != 0x0C) return false;
  for (uint32_t i = 0; i < n && r.ok; ++i) {
    std::string nm = r.name();
    int t = (int)r.u32();
    uint32_t cnt = r.u32();
    size_t bytes = cnt * type_size(t);
    if (!r.ok || r.pos + bytes > r.b.size()) return false;
    if (t == 2 && keep) keep->emplace_back(nm, r.b.substr(r.pos, cnt));
    r.pos += (bytes + 3) & ~(size_t)3;
  }
  return r.ok;
}

// ------------------------------------------------------------------- CDL
struct Lexer {
  const std::string &s;
  size_t i = 0;
  explicit Lexer(const std::string &t) : s(t) {}
  void skip() {
    for (;;) {
      while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
      if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '/') {
        while (i < s.size() && s[i] != '\n') ++i;
        continue;
      }
      break;
    }
  }
  // next token: word (identifier/number, ':' allowed inside), string, or one
  // punctuation character
  std::string next() {
    skip();
    if (i >= s.size()) return "";
    char c = s[i];
    if (c == '"') {
      size_t j = i + 1;
      while (j < s.size() && s[j] != '"') j += (s[j] == '\\') ? 2 : 1;
      std::string t = s.substr(i, j + 1 - i);
      i = j + 1;
      return t;
    }
    if (std::strchr("=,;(){}", c)) { ++i; return std::string(1, c); }
    size_t j = i;
    while (j < s.size() && !std::isspace((unsigned char)s[j]) && !std::strchr("=,;(){}\"", s[j])) ++j;
    std::string t = s.substr(i, j - i);
    i = j;
    return t;
  }
  std::string peek() {
    size_t k = i;
    std::string t = next();
    i = k;
    return t;
  }
};

int cdl_type(const std::string &w) {
  if (w == "byte") return 1;
  if (w == "char") return 2;
  if (w == "short") return 3;
  if (w == "int" || w == "long") return 4;
  if (w == "float" || w == "real") return 5;
  if (w == "double") return 6;
  return 0;
}

// A CDL number: C syntax, optional type suffix (1.5f, 3s, 2b, 1.0d), and
// Fortran-style D exponents.
bool parse_number(const std::string &w, double &v) {
  if (w.empty()) return false;
  std::string t = w;
  for (size_t k = 1; k + 1 < t.size(); ++k)
    if ((t[k] == 'D' || t[k] == 'd') && (std::isdigit((unsigned char)t[k - 1]) || t[k - 1] == '.') &&
        (t[k + 1] == '+' || t[k + 1] == '-' || std::isdigit((unsigned char)t[k + 1])))
      t[k] = 'E';
  char *end = nullptr;
  v = std::strtod(t.c_str(), &end);
  if (end == t.c_str()) return false;
  if (*end == '\0') return true;
  return end[1] == '\0' && std::strchr("fFdDsSbBlL", end[0]) != nullptr;
}

std::string format_e(double v) {
  char buf[32];
  std::snprintf(buf, sizeof(buf), "%13.6E", v);
  return buf;
}

const char *type_word(int t) {
  switch (t) {
    case 1: return "byte";
    case 2: return "char";
    case 3: return "short";
    case 4: return "int";
    case 6: return "double";
    default: return "float";
  }
}

void put32(std::string &o, uint32_t v) {
  o.push_back((char)(v >> 24)); o.push_back((char)(v >> 16)); o.push_back((char)(v >> 8)); o.push_back((char)v);
}

void put_name(std::string &o, const std::string &n) {
  put32(o, (uint32_t)n.size());
  o += n;
  while (o.size() % 4) o.push_back('\0');
}

void put_value(std::string &o, double v, int t) {
  switch (t) {
    case 4: put32(o, (uint32_t)(int32_t)std::llround(v)); break;
    case 6: {
      uint64_t u;
      std::memcpy(&u, &v, 8);
      put32(o, (uint32_t)(u >> 32));
      put32(o, (uint32_t)u);
      break;
    }
    default: {
      float f = (float)v;
      uint32_t u;
      std::memcpy(&u, &f, 4);
      put32(o, u);
    }
  }
}

}  // namespace

bool read_cdf(const std::string &path, NcFile &f, std::string &err) {
  std::string b;
  if (!slurp(path, b)) { err = "cannot open " + path; return false; }
  if (b.size() < 8 || b.compare(0, 3, "CDF") != 0 || (b[3] != 1 && b[3] != 2)) {
    err = path + " is not a netCDF classic file";
    return false;
  }
  const bool cdf2 = b[3] == 2;
  Reader r(b);
  r.pos = 4;
  const uint32_t numrecs = r.u32();
  f = NcFile{};
  f.name = path;
  // dimensions
  uint32_t tag = r.u32(), n = r.u32();
  int rec_dim = -1;
  if (tag == 0x0A) {
    for (uint32_t i = 0; i < n && r.ok; ++i) {
      std::string nm = r.name();
      uint32_t len = r.u32();
      if (len == 0) { rec_dim = (int)i; len = numrecs; }
      f.dims.emplace_back(nm, len);
    }
  } else if (!(tag == 0 && n == 0)) {
    err = path + ": bad dimension list";
    return false;
  }
  if (!read_atts(r, nullptr)) { err = path + ": bad global attributes"; return false; }
  // variables
  tag = r.u32();
  n = r.u32();
  struct Meta { size_t begin, vsize; bool rec; };
  std::vector<Meta> meta;
  if (tag == 0x0B) {
    for (uint32_t i = 0; i < n && r.ok; ++i) {
      NcVar v;
      v.name = r.name();
      uint32_t nd = r.u32();
      for (uint32_t k = 0; k < nd; ++k) v.dims.push_back((int)r.u32());
      if (!read_atts(r, &v.text_atts)) { err = path + ": bad attributes of " + v.name; return false; }
      v.type = (int)r.u32();
      size_t vsize = r.u32();
      size_t begin = cdf2 ? (size_t)r.u64() : (size_t)r.u32();
      meta.push_back({begin, vsize, !v.dims.empty() && v.dims[0] == rec_dim});
      f.vars.push_back(std::move(v));
    }
  } else if (!(tag == 0 && n == 0)) {
    err = path + ": bad variable list";
    return false;
  }
  if (!r.ok) { err = path + ": truncated header"; return false; }
  size_t recsize = 0;
  for (const Meta &m : meta)
    if (m.rec) recsize += m.vsize;
  for (size_t k = 0; k < f.vars.size(); ++k) {
    NcVar &v = f.vars[k];
    const size_t es = type_size(v.type);
    if (es == 0) { err = path + ": unknown type of " + v.name; return false; }
    size_t per_rec = 1, total = 1;
    for (size_t d = 0; d < v.dims.size(); ++d) {
      if (v.dims[d] < 0 || v.dims[d] >= (int)f.dims.size()) { err = path + ": bad dimension id"; return false; }
      const size_t len = f.dims[v.dims[d]].second;
      total *= len;
      if (!(meta[k].rec && d == 0)) per_rec *= len;
    }
    v.data.resize(total);
    if (meta[k].rec) {
      for (size_t rr = 0; rr < numrecs; ++rr)
        for (size_t q = 0; q < per_rec; ++q) {
          size_t at = meta[k].begin + rr * recsize + q * es;
          if (at + es > b.size()) { err = path + ": truncated data"; return false; }
          v.data[rr * per_rec + q] = get_value(b, at, v.type);
        }
    } else {
      for (size_t q = 0; q < total; ++q) {
        size_t at = meta[k].begin + q * es;
        if (at + es > b.size()) { err = path + ": truncated data"; return false; }
        v.data[q] = get_value(b, at, v.type);
      }
    }
  }
  return true;
}

bool write_cdf(const std::string &path, const NcFile &f, std::string &err) {
  // header with placeholder offsets, then the data of each variable
  auto header = [&](const std::vector<size_t> &begins) {
    std::string o = "CDF";
    o.push_back('\x01');
    put32(o, 0);
    if (f.dims.empty()) { put32(o, 0); put32(o, 0); }
    else {
      put32(o, 0x0A);
      put32(o, (uint32_t)f.dims.size());
      for (auto &d : f.dims) { put_name(o, d.first); put32(o, (uint32_t)d.second); }
    }
    put32(o, 0); put32(o, 0);                      // no global attributes
    if (f.vars.empty()) { put32(o, 0); put32(o, 0); }
    else {
      put32(o, 0x0B);
      put32(o, (uint32_t)f.vars.size());
      for (size_t k = 0; k < f.vars.size(); ++k) {
        const NcVar &v = f.vars[k];
        put_name(o, v.name);
        put32(o, (uint32_t)v.dims.size());
        for (int d : v.dims) put32(o, (uint32_t)d);
        if (v.text_atts.empty()) { put32(o, 0); put32(o, 0); }
        else {
          put32(o, 0x0C);
          put32(o, (uint32_t)v.text_atts.size());
          for (auto &a : v.text_atts) {
            put_name(o, a.first);
            put32(o, 2);
            put32(o, (uint32_t)a.second.size());
            o += a.second;
            while (o.size() % 4) o.push_back('\0');
          }
        }
        const int t = (v.type == 4 || v.type == 6) ? v.type : 5;
        put32(o, (uint32_t)t);
        size_t vs = v.data.size() * type_size(t);
        put32(o, (uint32_t)((vs + 3) & ~(size_t)3));
        put32(o, (uint32_t)begins[k]);
      }
    }
    return o;
  };
  std::vector<size_t> begins(f.vars.size(), 0);
  std::string h = header(begins);
  size_t off = h.size();
  for (size_t k = 0; k < f.vars.size(); ++k) {
    begins[k] = off;
    const int t = (f.vars[k].type == 4 || f.vars[k].type == 6) ? f.vars[k].type : 5;
    off += (f.vars[k].data.size() * type_size(t) + 3) & ~(size_t)3;
  }
  if (off > 0x7fffffffu) { err = "file too large for CDF-1"; return false; }
  std::string o = header(begins);
  for (const NcVar &v : f.vars) {
    const int t = (v.type == 4 || v.type == 6) ? v.type : 5;
    for (double x : v.data) put_value(o, x, t);
    while (o.size() % 4) o.push_back('\0');
  }
  std::ofstream out(path, std::ios::binary);
  if (!out) { err = "cannot write " + path; return false; }
  out.write(o.data(), (std::streamsize)o.size());
  return (bool)out;
}

bool read_cdl(const std::string &path, NcFile &f, std::string &err) {
  std::string text;
  if (!slurp(path, text)) { err = "cannot open " + path; return false; }
  f = NcFile{};
  Lexer lx(text);
  if (lx.next() != "netcdf") { err = path + " is not a CDL file"; return false; }
  f.name = lx.next();
  if (f.name == "{") f.name.clear();
  else if (lx.next() != "{") { err = path + ": expected '{'"; return false; }
  std::string section;
  for (;;) {
    std::string t = lx.next();
    if (t.empty()) { err = path + ": unexpected end"; return false; }
    if (t == "}") break;
    if (t == "dimensions:" || t == "variables:" || t == "data:") { section = t; continue; }
    if (section == "dimensions:") {
      if (t == "," || t == ";") continue;
      if (lx.next() != "=") { err = path + ": bad dimension " + t; return false; }
      std::string v = lx.next();
      size_t len = (v == "UNLIMITED" || v == "unlimited") ? 0 : (size_t)std::strtoull(v.c_str(), nullptr, 10);
      f.dims.emplace_back(t, len);
    } else if (section == "variables:") {
      if (t == ";") continue;
      const int ty = cdl_type(t);
      if (ty) {
        NcVar v;
        v.type = ty;
        v.name = lx.next();
        if (lx.peek() == "(") {
          lx.next();
          for (;;) {
            std::string d = lx.next();
            if (d == ")") break;
            if (d == ",") continue;
            int di = f.dim_index(d);
            if (di < 0) { err = path + ": unknown dimension " + d; return false; }
            v.dims.push_back(di);
          }
        }
        f.vars.push_back(std::move(v));
      } else {
        // attribute: var:att = values ;  (global when it starts with ':')
        size_t c = t.find(':');
        std::string vn = c == std::string::npos ? "" : t.substr(0, c), an = c == std::string::npos ? t : t.substr(c + 1);
        if (lx.next() != "=") { err = path + ": bad attribute " + t; return false; }
        std::string val;
        for (;;) {
          std::string w = lx.next();
          if (w == ";" || w.empty()) break;
          if (w.size() >= 2 && w.front() == '"') val += w.substr(1, w.size() - 2);
        }
        for (NcVar &v : f.vars)
          if (v.name == vn) v.text_atts.emplace_back(an, val);
      }
    } else if (section == "data:") {
      if (t == ";") continue;
      NcVar *v = nullptr;
      for (NcVar &x : f.vars)
        if (x.name == t) v = &x;
      if (lx.next() != "=") { err = path + ": bad data of " + t; return false; }
      std::vector<double> vals;
      for (;;) {
        std::string w = lx.next();
        if (w == ";" || w.empty()) break;
        if (w == ",") continue;
        double x;
        if (w.front() == '"') continue;
        if (w == "_") { vals.push_back(NAN); continue; }
        if (!parse_number(w, x)) { err = path + ": bad number '" + w + "' in " + t; return false; }
        vals.push_back(x);
      }
      if (v) v->data = std::move(vals);
    }
  }
  for (NcVar &v : f.vars) {
    size_t total = 1;
    for (int d : v.dims) total *= f.dims[d].second;
    if (v.type != 2 && v.data.size() != total && !(v.dims.empty() && v.data.size() == 1)) {
      err = path + ": " + v.name + " holds " + std::to_string(v.data.size()) + " values, its dimensions " +
            std::to_string(total);
      return false;
    }
  }
  return true;
}

bool write_cdl(const std::string &path, const NcFile &f, std::string &err) {
  std::ostringstream o;
  o << "netcdf " << (f.name.empty() ? "data" : f.name) << "{\n\ndimensions:\n";
  for (auto &d : f.dims) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "    %-15s= %3zu;\n", d.first.c_str(), d.second);
    o << buf;
  }
  o << "\n\nvariables:\n";
  for (const NcVar &v : f.vars) {
    o << "    " << type_word(v.type) << " " << v.name;
    if (!v.dims.empty()) {
      o << "(";
      for (size_t k = 0; k < v.dims.size(); ++k) o << (k ? "," : "") << f.dims[v.dims[k]].first;
      o << ")";
    }
    o << ";\n";
    for (auto &a : v.text_atts) o << "             " << v.name << ":" << a.first << " = \"" << a.second << "\";\n";
  }
  o << "\ndata:\n";
  for (const NcVar &v : f.vars) {
    char head[64];
    std::snprintf(head, sizeof(head), "%17s = ", v.name.c_str());
    o << head;
    for (size_t k = 0; k < v.data.size(); ++k) {
      if (k) o << (k % 4 == 0 ? ",\n                    " : ", ");
      if (v.type == 4) o << (long long)std::llround(v.data[k]);
      else o << format_e(v.data[k]);
    }
    o << ";\n";
  }
  o << "\n}\n";
  std::ofstream out(path);
  if (!out) { err = "cannot write " + path; return false; }
  out << o.str();
  return (bool)out;
}

bool read_nc(const std::string &path, NcFile &f, std::string &err) {
  std::ifstream in(path, std::ios::binary);
  if (!in) { err = "cannot open " + path; return false; }
  char m[3] = {0, 0, 0};
  in.read(m, 3);
  if (in.gcount() == 3 && m[0] == 'C' && m[1] == 'D' && m[2] == 'F') return read_cdf(path, f, err);
  return read_cdl(path, f, err);
}

}  // namespace socgpu
