// Input-file front-end of the reference's explicit driver and its result
// writer, as host code above the C ABI:
//  * JSON decks (src/explicit/main.C:125-1005): a deck is read into a host
//    object (mesh, material, the ordered list of AddBCVelNode calls, options,
//    time step) that can be inspected and then applied to a domain;
//  * LS-DYNA keyword meshes, *NODE and *ELEMENT_SOLID
//    (Domain_d::CreateFromLSDyna, Domain_d.C:1647-1699);
//  * Nastran GRID/CTRIA die meshes (NastranReader.cpp, Mesh.C:560-760);
//  * legacy VTK output (VTKWriter.C) of a domain's current state.
// Everything reaches the domain through the public wf_* entry points.
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "wf.h"
#include "wf_internal.cuh"

namespace {

// ---- JSON ---------------------------------------------------------------------
struct JVal {
  enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<JVal> arr;
  std::vector<std::pair<std::string, JVal>> obj;

  const JVal *get(const char *key) const {
    if (kind != Obj) return nullptr;
    for (const auto &kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
  const JVal *at(size_t i) const { return (kind == Arr && i < arr.size()) ? &arr[i] : nullptr; }
};

// Recursive-descent parser of RFC 8259 JSON (UTF-8 passed through; \u escapes
// of the Basic Multilingual Plane encoded as UTF-8). Nesting is limited.
class JParser {
 public:
  explicit JParser(const std::string &s) : s_(s) {}
  std::string err;

  bool parse(JVal &out) {
    ws();
    if (!value(out, 0)) return false;
    ws();
    if (i_ != s_.size()) return fail("trailing characters after the top-level value");
    return true;
  }

 private:
  const std::string &s_;
  size_t i_ = 0;
  int line_ = 1;

  bool fail(const std::string &m) {
    err = "line " + std::to_string(line_) + ": " + m;
    return false;
  }
  void ws() {
    while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) {
      if (s_[i_] == '\n') line_++;
      i_++;
    }
  }
  bool lit(const char *w) {
    const size_t n = std::strlen(w);
    if (s_.compare(i_, n, w) != 0) return false;
    i_ += n;
    return true;
  }
  bool value(JVal &v, int depth) {
    if (depth > 128) return fail("nesting too deep");
    if (i_ >= s_.size()) return fail("unexpected end of input");
    const char c = s_[i_];
    if (c == '{') return object(v, depth);
    if (c == '[') return array(v, depth);
    if (c == '"') {
      v.kind = JVal::Str;
      return string(v.str);
    }
    if (lit("true")) {
      v.kind = JVal::Bool;
      v.b = true;
      return true;
    }
    if (lit("false")) {
      v.kind = JVal::Bool;
      v.b = false;
      return true;
    }
    if (lit("null")) {
      v.kind = JVal::Null;
      return true;
    }
    return number(v);
  }
  bool number(JVal &v) {
    const size_t b = i_;
    if (i_ < s_.size() && (s_[i_] == '-' || s_[i_] == '+')) i_++;
    while (i_ < s_.size() &&
           (std::isdigit((unsigned char)s_[i_]) || s_[i_] == '.' || s_[i_] == 'e' ||
            s_[i_] == 'E' || s_[i_] == '-' || s_[i_] == '+'))
      i_++;
    if (i_ == b) return fail(std::string("unexpected character '") + s_[b] + "'");
    const std::string t = s_.substr(b, i_ - b);
    char *end = nullptr;
    v.num = std::strtod(t.c_str(), &end);
    if (!end || *end != '\0') return fail("malformed number '" + t + "'");
    v.kind = JVal::Num;
    return true;
  }
  static void utf8(std::string &o, unsigned cp) {
    if (cp < 0x80) {
      o += (char)cp;
    } else if (cp < 0x800) {
      o += (char)(0xC0 | (cp >> 6));
      o += (char)(0x80 | (cp & 0x3F));
    } else {
      o += (char)(0xE0 | (cp >> 12));
      o += (char)(0x80 | ((cp >> 6) & 0x3F));
      o += (char)(0x80 | (cp & 0x3F));
    }
  }
  bool string(std::string &o) {
    i_++;  // opening quote
    o.clear();
    while (i_ < s_.size()) {
      const char c = s_[i_++];
      if (c == '"') return true;
      if (c == '\n') return fail("newline inside a string");
      if (c != '\\') {
        o += c;
        continue;
      }
      if (i_ >= s_.size()) break;
      const char e = s_[i_++];
      switch (e) {
        case '"': o += '"'; break;
        case '\\': o += '\\'; break;
        case '/': o += '/'; break;
        case 'b': o += '\b'; break;
        case 'f': o += '\f'; break;
        case 'n': o += '\n'; break;
        case 'r': o += '\r'; break;
        case 't': o += '\t'; break;
        case 'u': {
          if (i_ + 4 > s_.size()) return fail("short \\u escape");
          unsigned cp = 0;
          for (int k = 0; k < 4; k++) {
            const char h = s_[i_++];
            cp <<= 4;
            if (h >= '0' && h <= '9') cp |= (unsigned)(h - '0');
            else if (h >= 'a' && h <= 'f') cp |= (unsigned)(h - 'a' + 10);
            else if (h >= 'A' && h <= 'F') cp |= (unsigned)(h - 'A' + 10);
            else return fail("bad \\u escape");
          }
          utf8(o, cp);
          break;
        }
        default: return fail(std::string("bad escape \\") + e);
      }
    }
    return fail("unterminated string");
  }
  bool array(JVal &v, int depth) {
    v.kind = JVal::Arr;
    i_++;
    ws();
    if (i_ < s_.size() && s_[i_] == ']') {
      i_++;
      return true;
    }
    for (;;) {
      v.arr.emplace_back();
      ws();
      if (!value(v.arr.back(), depth + 1)) return false;
      ws();
      if (i_ >= s_.size()) return fail("unterminated array");
      if (s_[i_] == ',') {
        i_++;
        continue;
      }
      if (s_[i_] == ']') {
        i_++;
        return true;
      }
      return fail("expected ',' or ']' in array");
    }
  }
  bool object(JVal &v, int depth) {
    v.kind = JVal::Obj;
    i_++;
    ws();
    if (i_ < s_.size() && s_[i_] == '}') {
      i_++;
      return true;
    }
    for (;;) {
      ws();
      if (i_ >= s_.size() || s_[i_] != '"') return fail("expected a member name");
      std::string key;
      if (!string(key)) return false;
      ws();
      if (i_ >= s_.size() || s_[i_] != ':') return fail("expected ':' after \"" + key + "\"");
      i_++;
      ws();
      v.obj.emplace_back(key, JVal());
      if (!value(v.obj.back().second, depth + 1)) return false;
      ws();
      if (i_ >= s_.size()) return fail("unterminated object");
      if (s_[i_] == ',') {
        i_++;
        continue;
      }
      if (s_[i_] == '}') {
        i_++;
        return true;
      }
      return fail("expected ',' or '}' in object");
    }
  }
};

// readValue / readVector of the reference driver: set only when present.
bool jnum(const JVal *o, const char *k, double &out) {
  const JVal *v = o ? o->get(k) : nullptr;
  if (!v) return false;
  if (v->kind == JVal::Num) out = v->num;
  else if (v->kind == JVal::Bool) out = v->b ? 1.0 : 0.0;
  else return false;
  return true;
}
bool jint(const JVal *o, const char *k, int &out) {
  double t;
  if (!jnum(o, k, t)) return false;
  out = (int)t;
  return true;
}
bool jbool(const JVal *o, const char *k, bool &out) {
  const JVal *v = o ? o->get(k) : nullptr;
  if (!v) return false;
  if (v->kind == JVal::Bool) out = v->b;
  else if (v->kind == JVal::Num) out = v->num != 0.0;
  else return false;
  return true;
}
bool jstr(const JVal *o, const char *k, std::string &out) {
  const JVal *v = o ? o->get(k) : nullptr;
  if (!v || v->kind != JVal::Str) return false;
  out = v->str;
  return true;
}
// Up to n numbers of an array member (missing entries keep their value).
bool jvec(const JVal *o, const char *k, double *out, int n) {
  const JVal *v = o ? o->get(k) : nullptr;
  if (!v || v->kind != JVal::Arr) return false;
  for (int i = 0; i < n && i < (int)v->arr.size(); i++)
    if (v->arr[i].kind == JVal::Num) out[i] = v->arr[i].num;
  return true;
}

bool read_file(const std::string &path, std::string &out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

std::string dir_of(const std::string &p) {
  const size_t k = p.find_last_of("/\\");
  return k == std::string::npos ? std::string() : p.substr(0, k + 1);
}

// ---- LS-DYNA keyword mesh -------------------------------------------------------
struct KMesh {
  std::vector<double> x;          // [3 nn]
  std::vector<int32_t> elnod;     // [ne npe]
  int npe = 0;
};

std::string trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) a++;
  while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
  return s.substr(a, b - a);
}

// Fields of a data card: comma-separated (free format) or the fixed columns
// given by `widths`; a fixed-column card whose fields do not parse falls back
// to whitespace separation.
std::vector<std::string> card_fields(const std::string &line, const std::vector<int> &widths) {
  std::vector<std::string> f;
  if (line.find(',') != std::string::npos) {
    std::stringstream ss(line);
    std::string t;
    while (std::getline(ss, t, ',')) f.push_back(trim(t));
    return f;
  }
  size_t pos = 0;
  bool ok = true;
  for (int w : widths) {
    if (pos >= line.size()) break;
    const std::string t = trim(line.substr(pos, w));
    if (!t.empty() && t.find(' ') != std::string::npos) ok = false;
    f.push_back(t);
    pos += w;
  }
  if (ok && pos >= line.size()) return f;
  if (ok && trim(line.substr(std::min(pos, line.size()))).empty()) return f;
  f.clear();
  std::stringstream ss(line);
  std::string t;
  while (ss >> t) f.push_back(t);
  return f;
}

bool to_long(const std::string &t, long long &v) {
  if (t.empty()) return false;
  char *end = nullptr;
  v = std::strtoll(t.c_str(), &end, 10);
  return end && *end == '\0';
}
bool to_double(const std::string &t, double &v) {
  if (t.empty()) {
    v = 0.0;
    return true;
  }
  char *end = nullptr;
  v = std::strtod(t.c_str(), &end);
  return end && *end == '\0';
}

// *NODE cards: nid (8), x y z (16 each), tc rc (8); *ELEMENT_SOLID cards:
// eid pid n1..n8 (8 each). Nodes are numbered in the order of their cards;
// an element whose n5..n8 are absent or all equal to n4 is a tetrahedron
// (the keyword format's degenerate-hexahedron convention). All elements must
// have the same node count.
bool read_lsdyna(const std::string &path, KMesh &m, std::string &err) {
  std::string text;
  if (!read_file(path, text)) {
    err = "cannot open " + path;
    return false;
  }
  std::stringstream in(text);
  std::string line, kw;
  std::vector<long long> nid;
  std::vector<std::array<long long, 8>> el;
  std::vector<int> elnpe;
  int lineno = 0;
  const std::vector<int> node_w = {8, 16, 16, 16, 8, 8};
  const std::vector<int> elem_w = {8, 8, 8, 8, 8, 8, 8, 8, 8, 8};
  while (std::getline(in, line)) {
    lineno++;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.empty() || line[0] == '$') continue;
    if (line[0] == '*') {
      std::string k = trim(line.substr(1));
      const size_t sp = k.find_first_of(" \t");
      if (sp != std::string::npos) k = k.substr(0, sp);
      for (auto &c : k) c = (char)std::toupper((unsigned char)c);
      kw = k;
      if (kw.rfind("ELEMENT_SOLID", 0) == 0 && kw != "ELEMENT_SOLID") {
        err = "unsupported keyword *" + kw + " (line " + std::to_string(lineno) + ")";
        return false;
      }
      continue;
    }
    if (trim(line).empty()) continue;
    if (kw == "NODE") {
      const auto f = card_fields(line, node_w);
      long long id;
      double xyz[3] = {0, 0, 0};
      if (f.empty() || !to_long(f[0], id)) {
        err = "bad *NODE card at line " + std::to_string(lineno);
        return false;
      }
      for (int k = 0; k < 3; k++)
        if (k + 1 < (int)f.size() && !to_double(f[k + 1], xyz[k])) {
          err = "bad coordinate at line " + std::to_string(lineno);
          return false;
        }
      nid.push_back(id);
      m.x.insert(m.x.end(), xyz, xyz + 3);
    } else if (kw == "ELEMENT_SOLID") {
      const auto f = card_fields(line, elem_w);
      std::array<long long, 8> n{};
      int cnt = 0;
      for (size_t k = 2; k < f.size() && cnt < 8; k++) {
        long long v;
        if (f[k].empty()) break;
        if (!to_long(f[k], v)) {
          err = "bad *ELEMENT_SOLID card at line " + std::to_string(lineno);
          return false;
        }
        if (v == 0) break;
        n[cnt++] = v;
      }
      if (cnt != 4 && cnt != 8) {
        err = "element with " + std::to_string(cnt) + " nodes at line " + std::to_string(lineno);
        return false;
      }
      int npe = cnt;
      if (cnt == 8 && n[4] == n[3] && n[5] == n[3] && n[6] == n[3] && n[7] == n[3]) npe = 4;
      el.push_back(n);
      elnpe.push_back(npe);
    }
  }
  if (nid.empty() || el.empty()) {
    err = path + ": no *NODE or *ELEMENT_SOLID data";
    return false;
  }
  m.npe = elnpe[0];
  for (int p : elnpe)
    if (p != m.npe) {
      err = "mixed tetrahedra and hexahedra are not supported";
      return false;
    }
  std::unordered_map<long long, int32_t> index;
  index.reserve(nid.size() * 2);
  for (size_t k = 0; k < nid.size(); k++)
    if (!index.emplace(nid[k], (int32_t)k).second) {
      err = "duplicate node id " + std::to_string(nid[k]);
      return false;
    }
  m.elnod.resize(el.size() * m.npe);
  for (size_t e = 0; e < el.size(); e++)
    for (int a = 0; a < m.npe; a++) {
      auto it = index.find(el[e][a]);
      if (it == index.end()) {
        err = "element " + std::to_string(e + 1) + " references unknown node " +
              std::to_string(el[e][a]);
        return false;
      }
      m.elnod[e * m.npe + a] = it->second;
    }
  return true;
}

// ---- Nastran bulk data (rigid die meshes) -----------------------------------------
// NastranReader::read (NastranReader.cpp:34-180): lines starting GRID are
// nodes and lines starting CTRIA elements, each read as a run of consecutive
// lines from the first one of its kind; fixed 8-column fields, the id in the
// second field and the values from the fourth (column 24) on.
struct NasMesh {
  std::vector<double> x;     // [3 nn]
  std::vector<int32_t> tri;  // [3 ne] node positions, file order
};

// The 8-column field at `pos` (shorter at the end of the line); false when the
// line ends before the field starts.
bool nas_field(const std::string &line, size_t pos, std::string &f) {
  if (pos > line.size()) return false;
  f = line.substr(pos, 8);
  return true;
}

// A real field: a Fortran D exponent reads as E, and a field with no exponent
// letter takes one before its first sign past the first column ("1.5-3").
double nas_real(std::string f) {
  for (char &c : f)
    if (c == 'D' || c == 'd') c = 'E';
  if (f.find('E') == std::string::npos && f.find('e') == std::string::npos)
    for (size_t k = 1; k < f.size(); k++)
      if (f[k] == '+' || f[k] == '-') {
        f.insert(k, "E");
        break;
      }
  return std::strtod(f.c_str(), nullptr);
}

wf_status read_nastran(const std::string &path, NasMesh &m, std::string &err) {
  std::ifstream in(path);
  if (!in) {
    err = "cannot open " + path;
    return WF_ERR_ARG;
  }
  std::vector<std::string> lines;
  std::string ln;
  long long first_node = -1, first_elem = -1, nnode = 0, nelem = 0;
  bool lines2d = false;
  while (std::getline(in, ln)) {
    if (ln.compare(0, 4, "GRID") == 0) {
      if (first_node < 0) first_node = (long long)lines.size();
      nnode++;
    } else if (ln.compare(0, 5, "CTRIA") == 0 || ln.compare(0, 5, "CBEAM") == 0 ||
               ln.compare(0, 4, "CBAR") == 0) {
      if (first_elem < 0) first_elem = (long long)lines.size();
      if (ln[1] == 'B') lines2d = true;
      nelem++;
    }
    lines.push_back(ln);
  }
  if (lines2d) {
    err = path + ": CBEAM/CBAR line meshes are 2-D rigid bodies (3-D only)";
    return WF_ERR_UNSUPPORTED;
  }
  if (nnode < 3 || nelem < 1) {
    err = path + ": no GRID nodes or CTRIA triangles";
    return WF_ERR_ARG;
  }
  if (first_node + nnode > (long long)lines.size() || first_elem + nelem > (long long)lines.size()) {
    err = path + ": GRID and CTRIA cards must each be consecutive lines";
    return WF_ERR_ARG;
  }
  std::map<int, int32_t> pos;  // node id -> position (the first card of an id wins)
  m.x.assign(3 * nnode, 0.0);
  std::string f;
  for (long long n = 0; n < nnode; n++) {
    const std::string &L = lines[first_node + n];
    if (!nas_field(L, 8, f)) {
      err = path + ": short GRID card: " + L;
      return WF_ERR_ARG;
    }
    pos.emplace(std::atoi(f.c_str()), (int32_t)n);
    for (int i = 0; i < 3; i++) {
      if (!nas_field(L, 24 + 8 * i, f)) {
        err = path + ": short GRID card: " + L;
        return WF_ERR_ARG;
      }
      m.x[3 * n + i] = nas_real(f);
    }
  }
  m.tri.assign(3 * nelem, 0);
  for (long long e = 0; e < nelem; e++) {
    const std::string &L = lines[first_elem + e];
    for (int a = 0; a < 3; a++) {
      if (!nas_field(L, 24 + 8 * a, f)) {
        err = path + ": short CTRIA card: " + L;
        return WF_ERR_ARG;
      }
      const int id = std::atoi(f.c_str());
      auto it = pos.find(id);
      if (it == pos.end()) {
        err = path + ": triangle " + std::to_string(e + 1) + " references unknown node " +
              std::to_string(id);
        return WF_ERR_ARG;
      }
      m.tri[3 * e + a] = it->second;
    }
  }
  return WF_OK;
}

// TriMesh_d(NastranReader&, flipnormals, orientNormals, orient_pt) (Mesh.C:560-760):
// flipnormals swaps each triangle's first two nodes. With an orientation point
// P, a triangle turns (first two nodes swapped again) when its normal points
// away from the interior point C + 2 |C - P| (C - P) / |C - P|, C the mean
// of the die's nodes: the normals end up facing P, the part's side.
void nas_orient(const NasMesh &m, bool flip, const double *P, std::vector<int32_t> &tri) {
  const size_t nn = m.x.size() / 3, ne = m.tri.size() / 3;
  const double *X = m.x.data();
  double C[3] = {0.0, 0.0, 0.0};
  for (size_t n = 0; n < nn; n++)
    for (int k = 0; k < 3; k++) C[k] = C[k] + X[3 * n + k];
  const double inv_nn = 1.0 / (double)nn;
  for (int k = 0; k < 3; k++) C[k] = C[k] * inv_nn;
  tri.resize(3 * ne);
  double S[3] = {0.0, 0.0, 0.0};
  if (P) {
    double dir[3] = {C[0] - P[0], C[1] - P[1], C[2] - P[2]};
    const double dist = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    const double inv = 1.0 / dist;
    for (int k = 0; k < 3; k++) dir[k] = dir[k] * inv;
    for (int k = 0; k < 3; k++) S[k] = C[k] + dir[k] * (2.0 * dist);
  }
  const double third = 1.0 / 3.;
  for (size_t e = 0; e < ne; e++) {
    const int32_t c0 = m.tri[3 * e], c1 = m.tri[3 * e + 1], c2 = m.tri[3 * e + 2];
    const double *p0 = &X[3 * c0], *p1 = &X[3 * c1], *p2 = &X[3 * c2];
    int32_t *t = &tri[3 * e];
    t[0] = flip ? c1 : c0;
    t[1] = flip ? c0 : c1;
    t[2] = c2;
    if (!P) continue;
    const double u[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    const double v[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    double w[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                   u[0] * v[1] - u[1] * v[0]};
    for (int pass = 0; pass < 2; pass++) {
      const double inv = 1.0 / std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
      for (int k = 0; k < 3; k++) w[k] = w[k] * inv;
    }
    if (flip)
      for (int k = 0; k < 3; k++) w[k] = -w[k];
    double g[3];
    for (int k = 0; k < 3; k++) g[k] = ((p0[k] + p1[k]) + p2[k]) * third - S[k];
    if (w[0] * g[0] + w[1] * g[1] + w[2] * g[2] < 0.0) std::swap(t[0], t[1]);
  }
}

// A file named in a deck: relative to the deck's folder when it exists there,
// else as given (relative to the working directory) or absolute.
std::string resolve(const std::string &deck, const std::string &fname) {
  if (!fname.empty() && fname[0] == '/') return fname;
  const std::string full = dir_of(deck) + fname;
  std::ifstream probe(full);
  return probe ? full : fname;
}

// TriMesh_d::AxisPlaneMesh for axis 2 (Mesh.C:48-200), the Plane rigid body:
// (dens+1)^2 nodes at z = start.z spaced (dim.x - start.x) / dens in x and y,
// two triangles per cell with normal +z, or -z with flipnormals.
void plane_mesh(const double *st, const double *dm, int dens, bool flip, std::vector<double> &x,
                std::vector<int32_t> &tri) {
  const double dl = (dm[0] - st[0]) / dens;
  double x2 = st[1];
  for (int jj = 0; jj <= dens; jj++) {
    double x1 = st[0];
    for (int ii = 0; ii <= dens; ii++) {
      x.push_back(x1);
      x.push_back(x2);
      x.push_back(st[2]);
      x1 += dl;
    }
    x2 += dl;
  }
  for (int jj = 0; jj < dens; jj++)
    for (int ii = 0; ii < dens; ii++) {
      const int32_t n0 = (dens + 1) * jj + ii, n1 = n0 + 1, n2 = (dens + 1) * (jj + 1) + ii,
                    n3 = n2 + 1;
      const int32_t t[2][3] = {{n0, n1, n2}, {n1, n3, n2}};
      const int32_t tf[2][3] = {{n0, n2, n1}, {n1, n2, n3}};
      for (int q = 0; q < 2; q++)
        for (int c = 0; c < 3; c++) tri.push_back(flip ? tf[q][c] : t[q][c]);
    }
}

// Domain_d::calcMinEdgeLength in 3-D (Domain_d.C:2224-2469): every element is
// read as a tetrahedron of its first four nodes and the six segments between
// them are measured.
double ref_min_length(const std::vector<double> &x, const std::vector<int32_t> &elnod, int npe) {
  double mn = 1.0e6;
  const size_t ne = elnod.size() / npe;
  for (size_t e = 0; e < ne; e++) {
    const int32_t *n = &elnod[e * npe];
    const int pr[6][2] = {{1, 0}, {2, 0}, {3, 0}, {2, 1}, {3, 1}, {3, 2}};
    for (const auto &p : pr) {
      const double dx = x[3 * n[p[0]]] - x[3 * n[p[1]]];
      const double dy = x[3 * n[p[0]] + 1] - x[3 * n[p[1]] + 1];
      const double dz = x[3 * n[p[0]] + 2] - x[3 * n[p[1]] + 2];
      const double len = std::sqrt(dx * dx + dy * dy + dz * dz);
      if (len < mn) mn = len;
    }
  }
  return mn;
}

}  // namespace

// ---- deck object ---------------------------------------------------------------------
// A rigid body of a contact deck: triangle mesh, zone id and the velocity the
// boundary condition of that zone gives it.
struct DeckBody {
  std::vector<double> x;
  std::vector<int32_t> tri;
  int zone = 0;
  double vel[3] = {0.0, 0.0, 0.0};
};

struct wf_deck {
  wf_deck_info info{};
  std::vector<DeckBody> bodies;
  std::vector<double> x;
  std::vector<int32_t> elnod;
  std::vector<int64_t> bc_node;
  std::vector<int32_t> bc_dim;
  std::vector<double> bc_val;
};

namespace {

wf_status deck_fail(char *err, int64_t len, const std::string &m, wf_status s = WF_ERR_ARG) {
  if (err && len > 0) {
    std::strncpy(err, m.c_str(), (size_t)len - 1);
    err[len - 1] = '\0';
  }
  return s;
}

}  // namespace

WF_API wf_status wf_deck_read(const char *path, wf_deck **out, char *err, int64_t err_len) {
  if (!path || !out) return WF_ERR_ARG;
  *out = nullptr;
  std::string text;
  if (!read_file(path, text)) return deck_fail(err, err_len, std::string("cannot open ") + path);
  JVal j;
  JParser jp(text);
  if (!jp.parse(j)) return deck_fail(err, err_len, std::string(path) + ": " + jp.err);
  if (j.kind != JVal::Obj) return deck_fail(err, err_len, "the deck is not a JSON object");
  wf_deck *k = new wf_deck();
  wf_deck_info &I = k->info;
  auto bad = [&](const std::string &m, wf_status s = WF_ERR_ARG) {
    delete k;
    return deck_fail(err, err_len, m, s);
  };
  const JVal *config = j.get("Configuration");
  const JVal *stab = j.get("Stabilization");
  const JVal *mats = j.get("Materials");
  const JVal *blocks = j.get("DomainBlocks");
  const JVal *zones = j.get("DomainZones");
  const JVal *bcs = j.get("BoundaryConditions");
  const JVal *rig = j.get("RigidBodies");

  // Configuration (main.C:214-330)
  I.cfl = 0.3;
  jnum(config, "simTime", I.end_time);
  jnum(config, "outTime", I.out_time);
  jnum(config, "cflFactor", I.cfl);
  jint(config, "pressAlgorithm", I.press_alg);
  if (I.press_alg < 0) I.press_alg = 0;
  // plastic heat fraction and strain-rate cap of the stress update (main.C:218, 228)
  I.plheat_frac = 0.9;
  I.max_edot = 1.0e6;
  jnum(config, "plHeatFrac", I.plheat_frac);
  jnum(config, "maxStrRate", I.max_edot);
  if (!(I.plheat_frac >= 0.0 && I.plheat_frac <= 1.0)) return bad("plHeatFrac not in [0, 1]");
  if (!(I.max_edot > 0.0)) return bad("maxStrRate must be > 0");
  {
    double av[3] = {0, 0, 0};
    jvec(config, "artifViscCoeffs", av, 3);
    I.artif_visc[0] = av[0];
    I.artif_visc[1] = av[1];
  }
  bool sym[3] = {false, false, false};
  double symtol = 1.0e-4;
  jbool(config, "xSymm", sym[0]);
  jbool(config, "ySymm", sym[1]);
  jbool(config, "zSymm", sym[2]);
  jnum(config, "symtol", symtol);
  // thermal coupling (main.C:424-441): InitialConditions Temp (last entry wins)
  bool thermal = false;
  jbool(config, "thermal", thermal);
  I.thermal = thermal ? 1 : 0;
  I.T0 = 20.0;
  if (const JVal *ics = j.get("InitialConditions"))
    if (ics->kind == JVal::Arr)
      for (const JVal &ic : ics->arr) jnum(&ic, "Temp", I.T0);
  std::string s;
  if (jstr(config, "plasticType", s) && s != "Hardening")
    return bad("plasticType " + s + " is not supported", WF_ERR_UNSUPPORTED);
  if (jstr(config, "domType", s) && s != "3D")
    return bad("domType " + s + " is not supported (3-D only)", WF_ERR_UNSUPPORTED);
  jnum(config, "hourglass3D", I.hourglass);

  // Stabilization (loadStabilizationParams, main.C:84-118)
  if (stab && stab->kind == JVal::Obj) {
    I.has_stab = 1;
    jnum(stab, "alpha_free", I.stab.alpha_free);
    jnum(stab, "alpha_contact", I.stab.alpha_contact);
    jnum(stab, "hg_coeff_free", I.stab.hg_coeff_free);
    jnum(stab, "hg_coeff_contact", I.stab.hg_coeff_contact);
    jnum(stab, "av_coeff_div", I.stab.av_coeff_div);
    jnum(stab, "av_coeff_bulk", I.stab.av_coeff_bulk);
    jnum(stab, "log_factor", I.stab.log_factor);
    jnum(stab, "p_pspg_bulkfac", I.stab.p_pspg_bulkfac);
    jnum(stab, "J_min", I.stab.J_min);
  }

  // Materials[0] (main.C:441-575)
  const JVal *m0 = mats ? mats->at(0) : nullptr;
  if (!m0) return bad("no Materials entry");
  wf_material &M = I.material;
  M = wf_material{};
  jnum(m0, "density0", M.rho);
  jnum(m0, "youngsModulus", M.E);
  jnum(m0, "poissonsRatio", M.nu);
  jnum(m0, "yieldStress0", M.sy0);
  double c[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  jvec(m0, "const", c, 10);
  std::string mtype = "Bilinear";
  jstr(m0, "type", mtype);
  if (!(M.E > 0.0) || !(M.rho > 0.0)) return bad("material needs youngsModulus > 0 and density0 > 0");
  if (mtype == "Bilinear") {
    // plastic modulus from the tangent modulus const[0] (main.C:489)
    M.model = WF_MAT_BILINEAR;
    M.H = M.E * c[0] / (M.E - c[0]);
  } else if (mtype == "Hollomon") {
    M.model = WF_MAT_HOLLOMON;
    M.hol_K = c[0];
    M.hol_m = c[1];
  } else if (mtype == "JohnsonCook") {
    // JohnsonCook(el, Fy, B, n, C, eps0_dot, m, T_m, T_t) from const (main.C:538-541):
    // m, T_m, T_t are const[4..6] with thermal coupling, else 1, 1e10, 0
    M.model = WF_MAT_JOHNSON_COOK;
    const double jc[8] = {c[0], c[1], c[2], c[3], thermal ? c[4] : 1.0, thermal ? c[5] : 1.0e10,
                          thermal ? c[6] : 0.0, thermal ? I.T0 : 0.0};
    for (int q = 0; q < 8; q++) I.johnson_cook[q] = jc[q];
  } else if (mtype == "GMT") {
    // GMT(el, n1, n2, C1, C2, m1, m2, I1, I2, e_range, er_range, T_range) from
    // const and strRange / strdotRange / tempRange, each range defaulting to
    // [0, 1e10] (main.C:466-493, 548-553)
    M.model = WF_MAT_GMT;
    for (int q = 0; q < 8; q++) I.gmt[q] = c[q];
    double er[2] = {0.0, 1.0e10}, rr[2] = {0.0, 1.0e10}, tr[2] = {0.0, 1.0e10};
    jvec(m0, "strRange", er, 2);
    jvec(m0, "strdotRange", rr, 2);
    jvec(m0, "tempRange", tr, 2);
    const double rg[6] = {er[0], er[1], rr[0], rr[1], tr[0], tr[1]};
    for (int q = 0; q < 6; q++) I.gmt_range[q] = rg[q];
    if (!(er[0] > 0.0))
      return bad("GMT needs strRange with a lower bound > 0 (at zero strain the law is 0 * inf)");
  } else if (mtype == "NortonHoff") {
    return bad("material type NortonHoff is not supported: the reference's stress update reads "
               "none of its constants", WF_ERR_UNSUPPORTED);
  } else {
    return bad("material type " + mtype + " is not supported", WF_ERR_UNSUPPORTED);
  }

  // thermal constants (main.C:575-577)
  jnum(m0, "thermalCond", I.thermal_k);
  jnum(m0, "thermalHeatCap", I.thermal_cp);
  jnum(m0, "thermalExp", I.thermal_exp);
  if (thermal && !(I.thermal_cp > 0.0))
    return bad("thermal coupling needs Materials[0].thermalHeatCap > 0");

  // DomainBlocks[0] (main.C:350-430)
  const JVal *b0 = blocks ? blocks->at(0) : nullptr;
  if (!b0) return bad("no DomainBlocks entry");
  std::string btype = "Box";
  jstr(b0, "type", btype);
  if (btype == "File") {
    std::string fname;
    if (!jstr(b0, "fileName", fname)) return bad("File block without fileName");
    const std::string ext = fname.substr(fname.find_last_of('.') + 1);
    if (ext != "k") return bad("mesh file " + fname + ": only LS-DYNA .k meshes are read",
                               WF_ERR_UNSUPPORTED);
    const std::string full = resolve(path, fname);
    KMesh km;
    std::string e;
    if (!read_lsdyna(full, km, e)) return bad(e);
    k->x.swap(km.x);
    k->elnod.swap(km.elnod);
    I.npe = km.npe;
  } else if (btype == "Box") {
    double L[3] = {0, 0, 0}, V[3] = {0, 0, 0}, dx = 0.06;
    jvec(b0, "dim", L, 3);
    jvec(b0, "start", V, 3);
    jnum(b0, "elemLength", dx);
    std::string et;
    jstr(b0, "elemType", et);
    const bool tet = et == "TriTet";
    if (!(L[2] > 0.0)) return bad("Box block: only 3-D boxes (dim[2] > 0)", WF_ERR_UNSUPPORTED);
    std::string e;
    if (!wf::box_mesh(V, L, dx / 2.0, tet, k->x, k->elnod, e)) return bad(e);
    I.npe = tet ? 4 : 8;
  } else {
    return bad("DomainBlocks type " + btype + " is not supported", WF_ERR_UNSUPPORTED);
  }
  I.nn = (int64_t)(k->x.size() / 3);
  I.ne = (int64_t)(k->elnod.size() / I.npe);

  // Rigid bodies (main.C:633-830): entry 0 and, when present, entry 1 (the
  // reference reads no further entries) become rigid triangle meshes
  const JVal *r0 = rig ? rig->at(0) : nullptr;
  std::string rtype;
  if (r0 && jstr(r0, "type", rtype)) {
    // Domain_d::ComputeCentroid (Domain_d.C:2733-2755): default orientation point
    double cen[3] = {0.0, 0.0, 0.0};
    for (int64_t a = 0; a < I.nn; a++)
      for (int q = 0; q < 3; q++) cen[q] += k->x[3 * a + q];
    for (int q = 0; q < 3; q++) cen[q] /= (double)I.nn;
    const size_t nb = std::min<size_t>(rig->arr.size(), 2);
    for (size_t b = 0; b < nb; b++) {
      const JVal *r = rig->at(b);
      DeckBody body;
      std::string bt;
      jstr(r, "type", bt);
      jint(r, "zoneId", body.zone);
      bool flip = false;
      jbool(r, "flipnormals", flip);
      if (bt == "Plane") {
        double st[3] = {0, 0, 0}, dm[3] = {0, 0, 0};
        jvec(r, "start", st, 3);
        jvec(r, "dim", dm, 3);
        int dens = 1;
        jint(r, "partSide", dens);
        if (dens < 1) return bad("RigidBodies partSide must be >= 1");
        plane_mesh(st, dm, dens, flip, body.x, body.tri);
      } else if (bt == "File") {
        std::string fname;
        if (!jstr(r, "fileName", fname)) return bad("File rigid body without fileName");
        bool orient = true;
        jbool(r, "orientNormals", orient);
        double opt[3] = {cen[0], cen[1], cen[2]};
        jvec(r, "orientPoint", opt, 3);
        NasMesh nm;
        std::string e;
        const wf_status rs = read_nastran(resolve(path, fname), nm, e);
        if (rs) return bad(e, rs);
        nas_orient(nm, flip, orient ? opt : nullptr, body.tri);
        body.x.swap(nm.x);
      } else if (bt == "Line") {
        return bad("rigid body type Line is 2-D (3-D only)", WF_ERR_UNSUPPORTED);
      } else {
        return bad("rigid body " + std::to_string(b) + ": type " + bt + " is not supported",
                   WF_ERR_UNSUPPORTED);
      }
      k->bodies.push_back(std::move(body));
    }
    I.contact = 1;
    I.rigid_bodies = (int32_t)k->bodies.size();
    I.die_nodes = (int32_t)(k->bodies[0].x.size() / 3);
    I.die_tris = (int32_t)(k->bodies[0].tri.size() / 3);
    I.penalty_factor = 0.1;  // Domain_d constructor (Domain_d.h:256)
    const JVal *c0 = j.get("Contact") ? j.get("Contact")->at(0) : nullptr;
    jnum(c0, "fricCoeffStatic", I.mu_static);
    jnum(c0, "fricCoeffDynamic", I.mu_dynamic);
    double pf = -1.0;
    if (jnum(c0, "penaltyFactor", pf) && pf > -1.0) I.penalty_factor = pf;
    // die heat transfer (main.C:714-719)
    I.die_temp = 20.0;
    jnum(c0, "heatCondCoeff", I.heat_cond);
    jnum(c0, "dieTemp", I.die_temp);
  } else if (rig && rig->kind == JVal::Arr && rig->arr.size() > 1) {
    return bad("a second rigid body needs a first one with a type");
  }

  // BoundaryConditions: AddBCVelZone per condition, in order (main.C:578-887)
  const double *X = k->x.data();
  auto add = [&](int64_t n, int d, double v) {
    k->bc_node.push_back(n);
    k->bc_dim.push_back(d);
    k->bc_val.push_back(v);
  };
  if (bcs && bcs->kind == JVal::Arr) {
    for (const JVal &bc : bcs->arr) {
      double st[3] = {0, 0, 0}, en[3] = {0, 0, 0}, val[3] = {0, 0, 0};
      jvec(&bc, "value", val, 3);
      if (I.contact) {
        // contact decks: the body's zone gives the die velocity and no zone
        // condition acts on the part (main.C:690-700, :737-750)
        int zid = -1;
        jint(&bc, "zoneId", zid);
        for (DeckBody &body : k->bodies)
          if (zid == body.zone)
            for (int q = 0; q < 3; q++) body.vel[q] = val[q];
        continue;
      }
      bool have = jvec(&bc, "start", st, 3) && jvec(&bc, "end", en, 3);
      if (!have) {
        // a condition without its own box takes the DomainZones entry of its zoneId
        int zid = -1;
        jint(&bc, "zoneId", zid);
        if (zones && zones->kind == JVal::Arr)
          for (const JVal &z : zones->arr) {
            int id = -2;
            jint(&z, "id", id);
            if (id == zid && jvec(&z, "start", st, 3) && jvec(&z, "end", en, 3)) {
              have = true;
              break;
            }
          }
        if (!have)
          return bad("boundary condition for zone " + std::to_string(zid) + " has no box");
      }
      I.n_zones++;
      for (int64_t a = 0; a < I.nn; a++) {
        const double *p = &X[3 * a];
        bool inside = true;
        for (int d = 0; d < 3; d++)
          if (p[d] < st[d] || p[d] > en[d]) inside = false;
        if (inside) {
          for (int d = 0; d < 3; d++) add(a, d, val[d]);
          I.zone_nodes++;
        }
      }
    }
  }
  if (I.contact)
    for (int q = 0; q < 3; q++) I.die_vel[q] = k->bodies[0].vel[q];
  // symmetry planes (main.C:945-960): coordinate < symtol fixes that dof
  for (int64_t a = 0; a < I.nn; a++)
    for (int d = 0; d < 3; d++)
      if (sym[d] && X[3 * a + d] < symtol) add(a, d, 0.0);
  I.n_bc = (int64_t)k->bc_node.size();

  // time step (main.C:862-879): dt = cflFactor * min length / sqrt(K / rho)
  const double K = M.E / (3.0 * (1.0 - 2.0 * M.nu));
  I.sound_speed = std::sqrt(K / M.rho);
  I.min_length = ref_min_length(k->x, k->elnod, I.npe);
  I.dt = I.cfl * I.min_length / I.sound_speed;
  *out = k;
  return WF_OK;
}

WF_API wf_status wf_deck_free(wf_deck *k) {
  delete k;
  return WF_OK;
}

WF_API wf_status wf_deck_get_info(const wf_deck *k, wf_deck_info *info) {
  if (!k || !info) return WF_ERR_ARG;
  *info = k->info;
  return WF_OK;
}

WF_API wf_status wf_deck_get_mesh(const wf_deck *k, double *xyz, int32_t *elnod) {
  if (!k) return WF_ERR_ARG;
  if (xyz) std::memcpy(xyz, k->x.data(), sizeof(double) * k->x.size());
  if (elnod) std::memcpy(elnod, k->elnod.data(), sizeof(int32_t) * k->elnod.size());
  return WF_OK;
}

WF_API wf_status wf_deck_get_die(const wf_deck *k, double *xyz, int32_t *tri) {
  if (!k) return WF_ERR_ARG;
  if (k->bodies.empty()) return WF_OK;
  const DeckBody &b = k->bodies[0];
  if (xyz) std::memcpy(xyz, b.x.data(), sizeof(double) * b.x.size());
  if (tri) std::memcpy(tri, b.tri.data(), sizeof(int32_t) * b.tri.size());
  return WF_OK;
}

WF_API wf_status wf_deck_get_body(const wf_deck *k, int32_t body, int64_t *nnodes, int64_t *ntris,
                                  double vel[3], double *xyz, int32_t *tri) {
  if (!k || body < 0 || body >= (int32_t)k->bodies.size()) return WF_ERR_ARG;
  const DeckBody &b = k->bodies[body];
  if (nnodes) *nnodes = (int64_t)(b.x.size() / 3);
  if (ntris) *ntris = (int64_t)(b.tri.size() / 3);
  if (vel)
    for (int q = 0; q < 3; q++) vel[q] = b.vel[q];
  if (xyz) std::memcpy(xyz, b.x.data(), sizeof(double) * b.x.size());
  if (tri) std::memcpy(tri, b.tri.data(), sizeof(int32_t) * b.tri.size());
  return WF_OK;
}

WF_API wf_status wf_read_nastran(const char *path, int32_t flip_normals, const double *orient_pt,
                                 double *xyz, int64_t cap_nodes, int32_t *tri, int64_t cap_tris,
                                 int64_t *nnodes, int64_t *ntris, char *err, int64_t err_len) {
  if (!path) return WF_ERR_ARG;
  NasMesh m;
  std::string e;
  const wf_status s = read_nastran(path, m, e);
  if (s) return deck_fail(err, err_len, e, s);
  std::vector<int32_t> t;
  nas_orient(m, flip_normals != 0, orient_pt, t);
  const int64_t nn = (int64_t)(m.x.size() / 3), ne = (int64_t)(t.size() / 3);
  if (nnodes) *nnodes = nn;
  if (ntris) *ntris = ne;
  if (xyz && cap_nodes > 0)
    std::memcpy(xyz, m.x.data(), sizeof(double) * 3 * (size_t)std::min(nn, cap_nodes));
  if (tri && cap_tris > 0)
    std::memcpy(tri, t.data(), sizeof(int32_t) * 3 * (size_t)std::min(ne, cap_tris));
  return WF_OK;
}

WF_API wf_status wf_deck_get_bcs(const wf_deck *k, int64_t *node, int32_t *dim, double *val) {
  if (!k) return WF_ERR_ARG;
  const size_t n = k->bc_node.size();
  if (node) std::memcpy(node, k->bc_node.data(), sizeof(int64_t) * n);
  if (dim) std::memcpy(dim, k->bc_dim.data(), sizeof(int32_t) * n);
  if (val) std::memcpy(val, k->bc_val.data(), sizeof(double) * n);
  return WF_OK;
}

WF_API wf_status wf_deck_apply(const wf_deck *k, wf_domain *d) {
  if (!k || !d) return WF_ERR_ARG;
  const wf_deck_info &I = k->info;
  wf_status s;
#define WF_DECK_TRY(call) \
  if ((s = (call)) != WF_OK) return s
  WF_DECK_TRY(wf_set_mesh(d, I.nn, I.ne, I.npe, k->x.data(), k->elnod.data()));
  WF_DECK_TRY(wf_set_materials(d, 1, &I.material));
  if (I.material.model == WF_MAT_JOHNSON_COOK) {
    const double *j = I.johnson_cook;
    WF_DECK_TRY(wf_set_johnson_cook(d, 0, j[0], j[1], j[2], j[3], j[4], j[5], j[6], j[7]));
  }
  if (I.material.model == WF_MAT_GMT)
    WF_DECK_TRY(wf_set_gmt(d, 0, I.gmt, I.gmt_range, I.thermal ? I.T0 : 0.0));
  WF_DECK_TRY(wf_set_density(d, I.material.rho));
  if (I.n_bc)
    WF_DECK_TRY(wf_add_bc_vel_nodes(d, I.n_bc, k->bc_node.data(), k->bc_dim.data(),
                                    k->bc_val.data()));
  WF_DECK_TRY(wf_allocate_bcs(d));
  if (I.has_stab) WF_DECK_TRY(wf_set_stab(d, &I.stab));
  if (I.press_alg) WF_DECK_TRY(wf_set_press_algorithm(d, I.press_alg));
  if (I.artif_visc[0] != 0.0 || I.artif_visc[1] != 0.0)
    WF_DECK_TRY(wf_set_artif_visc(d, I.artif_visc[0], I.artif_visc[1]));
  if (I.hourglass != 0.0) WF_DECK_TRY(wf_set_hourglass(d, I.hourglass));
  WF_DECK_TRY(wf_set_plastic_heat_fraction(d, I.plheat_frac));
  WF_DECK_TRY(wf_set_max_strain_rate(d, I.max_edot));
  if (I.thermal) {
    WF_DECK_TRY(wf_set_thermal(d, 1, I.T0));
    WF_DECK_TRY(wf_set_material_thermal(d, 0, I.thermal_k, I.thermal_cp, I.thermal_exp));
    if (I.contact) WF_DECK_TRY(wf_set_contact_heat(d, I.heat_cond, I.die_temp));
  }
  if (I.contact) {
    const DeckBody &b0 = k->bodies[0];
    WF_DECK_TRY(wf_set_contact_trimesh(d, I.die_nodes, b0.x.data(), I.die_tris, b0.tri.data(),
                                       b0.vel, I.mu_static, I.mu_dynamic, I.penalty_factor));
    for (size_t b = 1; b < k->bodies.size(); b++) {
      const DeckBody &bb = k->bodies[b];
      WF_DECK_TRY(wf_add_contact_trimesh(d, (int64_t)(bb.x.size() / 3), bb.x.data(),
                                         (int64_t)(bb.tri.size() / 3), bb.tri.data(), bb.vel));
    }
  }
  WF_DECK_TRY(wf_set_dt(d, I.dt));
  WF_DECK_TRY(wf_set_end_time(d, I.end_time));
#undef WF_DECK_TRY
  return WF_OK;
}

WF_API wf_status wf_load_deck(wf_domain *d, const char *path, wf_deck_info *info, char *err,
                              int64_t err_len) {
  if (!d || !path) return WF_ERR_ARG;
  wf_deck *k = nullptr;
  wf_status s = wf_deck_read(path, &k, err, err_len);
  if (s) return s;
  s = wf_deck_apply(k, d);
  if (s == WF_OK && info) *info = k->info;
  if (s && err && err_len > 0) deck_fail(err, err_len, wf_last_error(d), s);
  wf_deck_free(k);
  return s;
}

WF_API wf_status wf_load_lsdyna(wf_domain *d, const char *path) {
  if (!d || !path) return WF_ERR_ARG;
  KMesh km;
  std::string e;
  if (!read_lsdyna(path, km, e)) return wf::domain_fail(d, WF_ERR_ARG, e);
  return wf_set_mesh(d, (int64_t)km.x.size() / 3, (int64_t)km.elnod.size() / km.npe, km.npe,
                     km.x.data(), km.elnod.data());
}

// ---- VTK -------------------------------------------------------------------------
// Legacy ASCII unstructured grid of the current state with the field names of
// the reference's VTKWriter (VTKWriter.C:246-650): point data DISP, Velocity,
// Acceleration, nod_mass, ContForce and, with thermal coupling, Temp; cell data
// pressure, pl_strain, Vol, Rho, sigy and the stress tensor SIGMA.
// The reference's legacy VTK layout (VTKWriter::VTKWriter, VTKWriter.C:238-664):
// the part's nodes and elements, then the rigid triangle meshes as extra
// points and triangle cells; point data Position, DISP, Acceleration,
// Velocity, Part_ID, Temp (thermal), ContForce, nod_mass, stress (von Mises of
// the node-averaged stress), ext_nodes, nod_area, nod_p, SIGMAT (node-averaged
// stress) and EPSR (node-averaged strain rate, when kept); cell data ele_area,
// pressure, pl_strain, DDEVT (strain rate, when kept), J, Vol, Rho, Vol_0,
// sigy. Node averages are plain means over the node's elements, summed in
// element order (the reference's avgScalar). Tensors are written as the
// reference writes them, upper triangle with zeros below. Die points and
// triangles carry zeros (Part_ID 1, Temp the die temperature). Values are
// printed with 9 significant digits.
bool wf::write_vtk_text(const char *path, const wf::VtkView &v) {
  const int64_t nn = v.nn, ne = v.ne, tn = v.tri_nn, te = v.tri_ne, npe = v.npe;
  FILE *f = std::fopen(path, "w");
  if (!f) return false;
  auto ten = [&](const double *t, bool soa, int64_t i, int64_t n, int c) {
    return soa ? t[c * n + i] : t[6 * i + c];
  };
  // node averages of a 6-component element field, element order
  auto node_avg = [&](const double *t, bool soa, std::vector<double> &out) {
    out.assign(6 * nn, 0.0);
    std::vector<int32_t> cnt(nn, 0);
    for (int64_t e = 0; e < ne; e++)
      for (int64_t q = 0; q < npe; q++) {
        const int32_t n = v.elnod[e * npe + q];
        for (int c = 0; c < 6; c++) out[6 * n + c] += ten(t, soa, e, ne, c);
        cnt[n]++;
      }
    for (int64_t n = 0; n < nn; n++)
      if (cnt[n] > 0)
        for (int c = 0; c < 6; c++) out[6 * n + c] /= cnt[n];
  };
  std::fprintf(f, "# vtk DataFile Version 3.0\nweldform-gb300 results\nASCII\n"
                  "DATASET UNSTRUCTURED_GRID\nPOINTS %lld double\n", (long long)(nn + tn));
  for (int64_t n = 0; n < nn; n++)
    std::fprintf(f, "%.17g %.17g %.17g\n", v.x[3 * n], v.x[3 * n + 1], v.x[3 * n + 2]);
  for (int64_t n = 0; n < tn; n++)
    std::fprintf(f, "%.17g %.17g %.17g\n", v.tri_x[3 * n], v.tri_x[3 * n + 1],
                 v.tri_x[3 * n + 2]);
  std::fprintf(f, "CELLS %lld %lld\n", (long long)(ne + te), (long long)(ne * (npe + 1) + 4 * te));
  for (int64_t e = 0; e < ne; e++) {
    std::fprintf(f, "%d", (int)npe);
    for (int64_t q = 0; q < npe; q++) std::fprintf(f, " %d", v.elnod[e * npe + q]);
    std::fprintf(f, "\n");
  }
  for (int64_t e = 0; e < te; e++)
    std::fprintf(f, "3 %lld %lld %lld\n", (long long)(v.tri_el[3 * e] + nn),
                 (long long)(v.tri_el[3 * e + 1] + nn), (long long)(v.tri_el[3 * e + 2] + nn));
  std::fprintf(f, "CELL_TYPES %lld\n", (long long)(ne + te));
  for (int64_t e = 0; e < ne; e++) std::fprintf(f, "%d\n", npe == 8 ? 12 : 10);
  for (int64_t e = 0; e < te; e++) std::fprintf(f, "5\n");
  std::fprintf(f, "POINT_DATA %lld\n", (long long)(nn + tn));
  auto vec = [&](const char *name, const double *w) {
    std::fprintf(f, "VECTORS %s double\n", name);
    for (int64_t n = 0; n < nn; n++)
      std::fprintf(f, "%.9g %.9g %.9g\n", w[3 * n], w[3 * n + 1], w[3 * n + 2]);
    for (int64_t n = 0; n < tn; n++) std::fprintf(f, "0 0 0\n");
  };
  // scalar per node (w null: zeros) with the die points' value after it
  auto nscal = [&](const char *name, const double *w, double die) {
    std::fprintf(f, "SCALARS %s double 1\nLOOKUP_TABLE default\n", name);
    for (int64_t n = 0; n < nn; n++) std::fprintf(f, "%.9g\n", w ? w[n] : 0.0);
    for (int64_t n = 0; n < tn; n++) std::fprintf(f, "%.9g\n", die);
  };
  auto tens = [&](const char *name, const std::vector<double> &t, int64_t count, int64_t dummies) {
    std::fprintf(f, "TENSORS %s double\n", name);
    for (int64_t i = 0; i < count; i++) {
      const double *q = &t[6 * i];  // xx yy zz xy yz xz
      std::fprintf(f, "%.9g %.9g %.9g\n0 %.9g %.9g\n0 0 %.9g\n", q[0], q[3], q[5], q[1], q[4],
                   q[2]);
    }
    for (int64_t i = 0; i < dummies; i++) std::fprintf(f, "0 0 0\n0 0 0\n0 0 0\n");
  };
  vec("Position", v.x);
  vec("DISP", v.u);
  vec("Acceleration", v.a);
  vec("Velocity", v.v);
  nscal("Part_ID", nullptr, 1.0);
  if (v.T) nscal("Temp", v.T, v.T_die);
  vec("ContForce", v.cf);
  nscal("nod_mass", v.mass, 0.0);
  std::vector<double> avg;
  node_avg(v.sig, v.sig_soa, avg);
  {
    std::vector<double> seq(nn);
    for (int64_t n = 0; n < nn; n++) {
      const double *s6 = &avg[6 * n];
      const double tr = (s6[0] + s6[1] + s6[2]) / 3.0;
      const double dx = s6[0] - tr, dy = s6[1] - tr, dz = s6[2] - tr;
      const double J2 = 0.5 * (dx * dx + 2.0 * s6[3] * s6[3] + 2.0 * s6[5] * s6[5] + dy * dy +
                               2.0 * s6[4] * s6[4] + dz * dz);
      seq[n] = std::sqrt(3.0 * J2);
    }
    nscal("stress", seq.data(), 0.0);
  }
  {
    std::vector<double> ext(nn, 0.0);
    if (v.ext)
      for (int64_t n = 0; n < nn; n++) ext[n] = v.ext[n] ? 1.0 : 0.0;
    nscal("ext_nodes", ext.data(), 0.0);
  }
  nscal("nod_area", v.area, 0.0);
  {
    // calcNodalPressureFromElemental (Mechanical.C:1187-1213): volume-weighted
    // mean of the element pressures, element order
    std::vector<double> pn(nn, 0.0), wsum(nn, 0.0);
    for (int64_t e = 0; e < ne; e++)
      for (int64_t q = 0; q < npe; q++) {
        const int32_t n = v.elnod[e * npe + q];
        pn[n] += v.p[e] * v.vol[e];
        wsum[n] += v.vol[e];
      }
    for (int64_t n = 0; n < nn; n++)
      if (wsum[n] > 0.0) pn[n] /= wsum[n];
    nscal("nod_p", pn.data(), 0.0);
  }
  tens("SIGMAT", avg, nn, tn);
  if (v.sr) {
    node_avg(v.sr, v.sr_soa, avg);
    tens("EPSR", avg, nn, tn);
  }
  std::fprintf(f, "CELL_DATA %lld\n", (long long)(ne + te));
  auto escal = [&](const char *name, const double *w) {
    std::fprintf(f, "SCALARS %s double 1\nLOOKUP_TABLE default\n", name);
    for (int64_t e = 0; e < ne; e++) std::fprintf(f, "%.9g\n", w ? w[e] : 0.0);
    for (int64_t e = 0; e < te; e++) std::fprintf(f, "0\n");
  };
  escal("ele_area", nullptr);
  escal("pressure", v.p);
  escal("pl_strain", v.pl);
  if (v.sr) {
    std::vector<double> d6(6 * ne);
    for (int64_t e = 0; e < ne; e++)
      for (int c = 0; c < 6; c++) d6[6 * e + c] = ten(v.sr, v.sr_soa, e, ne, c);
    tens("DDEVT", d6, ne, te);
  }
  {
    std::vector<double> J(ne);
    for (int64_t e = 0; e < ne; e++) J[e] = v.vol[e] / v.vol0[e];
    escal("J", J.data());
  }
  escal("Vol", v.vol);
  escal("Rho", v.rho);
  escal("Vol_0", v.vol0);
  escal("sigy", v.sy);
  return std::fclose(f) == 0;
}
