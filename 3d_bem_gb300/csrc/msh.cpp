// msh.cpp -- mesh input on the host side of the boundary: GMSH ASCII meshes
// (format 2.2, as mshReader::readSections reads it, mshreader.cpp:200-376,
// and format 4.1), the include / exclude selection of elements by physical
// group name and geometric number (mshReader::sortOutIncludesAndExcludes /
// elementIsIncluded, :22-198 and :378-428), the split of quadrilaterals into
// triangles (global::quadrilateralsToTriangles, global.cpp:841-870) and the
// wall-impedance Robin data (WallImpedanceSection::setUpValues,
// SolvingScript/wallimpedancesection.cpp:308-405).
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/bemgpu.h"

namespace {

struct MshElem {
  int32_t type;    // 2 triangle, 3 quadrilateral
  int64_t node[4];
  int64_t phys, geom;
};

struct Interval {
  uint64_t lo, hi;
};

// Sorted, disjoint, non-adjacent intervals.
std::vector<Interval> normalise(std::vector<Interval> v) {
  for (Interval& i : v)
    if (i.lo > i.hi) std::swap(i.lo, i.hi);
  std::sort(v.begin(), v.end(), [](const Interval& a, const Interval& b) { return a.lo < b.lo; });
  std::vector<Interval> out;
  for (const Interval& i : v) {
    if (!out.empty() && (i.lo <= out.back().hi || i.lo - out.back().hi == 1))
      out.back().hi = std::max(out.back().hi, i.hi);
    else
      out.push_back(i);
  }
  return out;
}

// a minus b, both normalised
std::vector<Interval> difference(const std::vector<Interval>& a, const std::vector<Interval>& b) {
  std::vector<Interval> out;
  for (Interval cur : a) {
    bool alive = true;
    for (const Interval& e : b) {
      if (e.hi < cur.lo || e.lo > cur.hi) continue;
      if (e.lo > cur.lo) out.push_back({cur.lo, e.lo - 1});
      if (e.hi >= cur.hi) {
        alive = false;
        break;
      }
      cur.lo = e.hi + 1;
    }
    if (alive) out.push_back(cur);
  }
  return out;
}

bool in_intervals(uint64_t v, const std::vector<Interval>& iv) {
  for (const Interval& i : iv)
    if (v >= i.lo && v <= i.hi) return true;
  return false;
}

std::string lower(std::string s) {
  for (char& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

std::string strip_quotes(std::string s) {
  s.erase(std::remove(s.begin(), s.end(), '"'), s.end());
  s.erase(std::remove(s.begin(), s.end(), '\''), s.end());
  return s;
}

bool all_digits(const std::string& s) {
  return !s.empty() && std::all_of(s.begin(), s.end(), [](char c) { return c >= '0' && c <= '9'; });
}

// "a..b" / "a...b" with optional ends (the reference's range pattern
// ^(\d*)\.\.\.?(\d*)$): empty start = 1, empty end = unbounded
bool parse_range(const std::string& t, Interval& out, bool& empty) {
  const size_t p = t.find("..");
  if (p == std::string::npos) return false;
  std::string a = t.substr(0, p), b = t.substr(p + 2);
  if (!b.empty() && b[0] == '.') b = b.substr(1);
  if (!(a.empty() || all_digits(a)) || !(b.empty() || all_digits(b))) return false;
  empty = a.empty() && b.empty();
  out.lo = a.empty() ? 1 : std::strtoull(a.c_str(), nullptr, 10);
  out.hi = b.empty() ? std::numeric_limits<uint64_t>::max() : std::strtoull(b.c_str(), nullptr, 10);
  return true;
}

std::vector<std::string> split_list(const char* s) {
  std::vector<std::string> out;
  if (!s) return out;
  std::string cur;
  for (const char* p = s;; p++) {
    const char c = *p;
    if (c == 0 || std::isspace((unsigned char)c) || c == ',' || c == ';') {
      if (!cur.empty()) out.push_back(strip_quotes(cur));
      cur.clear();
      if (c == 0) break;
    } else {
      cur.push_back(c);
    }
  }
  out.erase(std::remove(out.begin(), out.end(), std::string()), out.end());
  return out;
}

// Line-oriented cursor over the file contents.
struct Cursor {
  const std::string& s;
  size_t pos = 0;
  explicit Cursor(const std::string& text) : s(text) {}
  bool eof() const { return pos >= s.size(); }
  std::string line() {
    const size_t e = s.find('\n', pos);
    std::string l = s.substr(pos, (e == std::string::npos ? s.size() : e) - pos);
    pos = e == std::string::npos ? s.size() : e + 1;
    if (!l.empty() && l.back() == '\r') l.pop_back();
    return l;
  }
  // next whitespace-separated token (crosses lines)
  bool token(std::string& t) {
    while (pos < s.size() && std::isspace((unsigned char)s[pos])) pos++;
    if (pos >= s.size()) return false;
    const size_t b = pos;
    while (pos < s.size() && !std::isspace((unsigned char)s[pos])) pos++;
    t.assign(s, b, pos - b);
    return true;
  }
  int64_t integer() {
    std::string t;
    if (!token(t)) throw std::string("unexpected end of file");
    char* end = nullptr;
    const long long v = std::strtoll(t.c_str(), &end, 10);
    if (end == t.c_str() || *end) throw "bad integer '" + t + "'";
    return (int64_t)v;
  }
  double real() {
    std::string t;
    if (!token(t)) throw std::string("unexpected end of file");
    char* end = nullptr;
    const double v = std::strtod(t.c_str(), &end);
    if (end == t.c_str() || *end) throw "bad number '" + t + "'";
    return v;
  }
  void rest_of_line() {
    while (pos < s.size() && s[pos] != '\n') pos++;
    if (pos < s.size()) pos++;
  }
  void expect_end(const char* tag) {
    std::string t;
    if (!token(t) || lower(t) != lower(tag)) throw std::string("missing ") + tag;
  }
};

}  // namespace

struct bem_msh {
  double version = 0;
  std::vector<double> xyz;                      // node coordinates, by index
  std::unordered_map<int64_t, int64_t> node_at; // node tag -> index
  std::vector<MshElem> elems;                   // triangles and quadrilaterals, file order
  std::vector<int32_t> pdim, ptag;
  std::vector<std::string> pname;
  std::vector<int64_t> sel_tri, sel_quad;       // current selection (indices into elems)
};

namespace {

void add_node(bem_msh& m, int64_t tag, double x, double y, double z) {
  m.node_at[tag] = (int64_t)(m.xyz.size() / 3);
  m.xyz.push_back(x);
  m.xyz.push_back(y);
  m.xyz.push_back(z);
}

// format 2.2: $Nodes, $Elements (number type ntags tags... nodes...), $PhysicalNames
void read_v2_nodes(Cursor& c, bem_msh& m) {
  const int64_t n = c.integer();
  if (n < 0) throw std::string("bad node count");
  m.xyz.reserve(m.xyz.size() + 3 * (size_t)n);
  for (int64_t i = 0; i < n; i++) {
    const int64_t tag = c.integer();
    const double x = c.real(), y = c.real(), z = c.real();
    add_node(m, tag, x, y, z);
  }
  c.expect_end("$EndNodes");
}

void read_v2_elements(Cursor& c, bem_msh& m) {
  const int64_t n = c.integer();
  if (n < 0) throw std::string("bad element count");
  c.rest_of_line();
  for (int64_t i = 0; i < n; i++) {
    const std::string l = c.line();
    std::vector<int64_t> v;
    const char* p = l.c_str();
    while (*p) {
      char* end = nullptr;
      const long long x = std::strtoll(p, &end, 10);
      if (end == p) break;
      v.push_back((int64_t)x);
      p = end;
    }
    if (v.size() < 3) throw std::string("short element line");
    const int64_t type = v[1], ntags = v[2];
    if (ntags < 0 || (int64_t)v.size() < 3 + ntags) throw std::string("bad element tags");
    const int nn = type == 2 ? 3 : (type == 3 ? 4 : 0);
    if (nn == 0) continue;  // lines, points, volume elements
    if ((int64_t)v.size() < 3 + ntags + nn) throw std::string("short element line");
    MshElem e{};
    e.type = (int32_t)type;
    e.phys = ntags >= 1 ? v[3] : 0;
    e.geom = ntags >= 2 ? v[4] : 0;
    for (int k = 0; k < nn; k++) e.node[k] = v[3 + ntags + k];
    m.elems.push_back(e);
  }
  c.expect_end("$EndElements");
}

void read_physical_names(Cursor& c, bem_msh& m) {
  const int64_t n = c.integer();
  c.rest_of_line();
  for (int64_t i = 0; i < n; i++) {
    const std::string l = c.line();
    int dim = 0, tag = 0, off = 0;
    if (std::sscanf(l.c_str(), "%d %d %n", &dim, &tag, &off) < 2)
      throw std::string("bad physical name line");
    std::string name = l.substr((size_t)off);
    while (!name.empty() && std::isspace((unsigned char)name.back())) name.pop_back();
    m.pdim.push_back(dim);
    m.ptag.push_back(tag);
    m.pname.push_back(strip_quotes(name));
  }
  c.expect_end("$EndPhysicalNames");
}

// format 4.1: $Entities (physical tags of each entity), block-structured
// $Nodes and $Elements; an element's geometric number is its entity tag, its
// physical number the entity's first physical tag (0 if none)
using EntityKey = int64_t;
EntityKey ekey(int64_t dim, int64_t tag) { return dim * (int64_t(1) << 40) + tag; }

void read_v4_entities(Cursor& c, std::unordered_map<EntityKey, int64_t>& phys) {
  const int64_t np = c.integer(), nc = c.integer(), ns = c.integer(), nv = c.integer();
  for (int64_t i = 0; i < np; i++) {
    const int64_t tag = c.integer();
    c.real(); c.real(); c.real();
    const int64_t k = c.integer();
    for (int64_t j = 0; j < k; j++) {
      const int64_t t = c.integer();
      if (j == 0) phys[ekey(0, tag)] = t;
    }
  }
  const int64_t counts[3] = {nc, ns, nv};
  for (int dim = 1; dim <= 3; dim++) {
    for (int64_t i = 0; i < counts[dim - 1]; i++) {
      const int64_t tag = c.integer();
      for (int q = 0; q < 6; q++) c.real();
      const int64_t k = c.integer();
      for (int64_t j = 0; j < k; j++) {
        const int64_t t = c.integer();
        if (j == 0) phys[ekey(dim, tag)] = t;
      }
      const int64_t nb = c.integer();
      for (int64_t j = 0; j < nb; j++) c.integer();
    }
  }
  c.expect_end("$EndEntities");
}

void read_v4_nodes(Cursor& c, bem_msh& m) {
  const int64_t nblocks = c.integer(), nnodes = c.integer();
  c.integer();
  c.integer();
  m.xyz.reserve(m.xyz.size() + 3 * (size_t)std::max<int64_t>(nnodes, 0));
  for (int64_t b = 0; b < nblocks; b++) {
    c.integer();  // entity dim
    c.integer();  // entity tag
    const int64_t parametric = c.integer(), n = c.integer();
    if (parametric != 0) throw std::string("parametric nodes are not supported");
    std::vector<int64_t> tags((size_t)n);
    for (int64_t i = 0; i < n; i++) tags[(size_t)i] = c.integer();
    for (int64_t i = 0; i < n; i++) {
      const double x = c.real(), y = c.real(), z = c.real();
      add_node(m, tags[(size_t)i], x, y, z);
    }
  }
  c.expect_end("$EndNodes");
}

int nodes_of_type(int64_t type) {
  switch (type) {  // GMSH element types (first-order and the common higher ones)
    case 1: return 2;
    case 2: return 3;
    case 3: return 4;
    case 4: return 4;
    case 5: return 8;
    case 6: return 6;
    case 7: return 5;
    case 8: return 3;
    case 9: return 6;
    case 10: return 9;
    case 11: return 10;
    case 15: return 1;
    case 16: return 8;
    default: return -1;
  }
}

void read_v4_elements(Cursor& c, bem_msh& m, const std::unordered_map<EntityKey, int64_t>& phys) {
  const int64_t nblocks = c.integer();
  c.integer();
  c.integer();
  c.integer();
  for (int64_t b = 0; b < nblocks; b++) {
    const int64_t dim = c.integer(), etag = c.integer(), type = c.integer(), n = c.integer();
    const int nn = nodes_of_type(type);
    if (nn < 0) throw "unsupported element type " + std::to_string(type);
    const auto it = phys.find(ekey(dim, etag));
    const int64_t ph = it == phys.end() ? 0 : it->second;
    for (int64_t i = 0; i < n; i++) {
      c.integer();  // element tag
      MshElem e{};
      e.type = (int32_t)type;
      e.phys = ph;
      e.geom = etag;
      for (int k = 0; k < nn; k++) {
        const int64_t t = c.integer();
        if (k < 4) e.node[k] = t;
      }
      if (type == 2 || type == 3) m.elems.push_back(e);
    }
  }
  c.expect_end("$EndElements");
}

void parse(const std::string& text, bem_msh& m) {
  Cursor c(text);
  std::unordered_map<EntityKey, int64_t> phys;
  bool have_format = false, have_nodes = false, have_elements = false;
  std::string t;
  while (c.token(t)) {
    const std::string tag = lower(t);
    if (tag == "$meshformat") {
      m.version = c.real();
      const int64_t file_type = c.integer();
      c.integer();  // data size
      if (file_type != 0) throw std::string("binary .msh files are not supported");
      if (!((m.version >= 2.0 && m.version < 3.0) || (m.version >= 4.1 && m.version < 5.0)))
        throw "unsupported .msh version " + std::to_string(m.version);
      c.expect_end("$EndMeshFormat");
      have_format = true;
    } else if (tag == "$physicalnames") {
      read_physical_names(c, m);
    } else if (tag == "$entities" && m.version >= 4.0) {
      read_v4_entities(c, phys);
    } else if (tag == "$nodes") {
      if (!have_format) throw std::string("$Nodes before $MeshFormat");
      if (m.version >= 4.0) read_v4_nodes(c, m);
      else read_v2_nodes(c, m);
      have_nodes = true;
    } else if (tag == "$elements") {
      if (!have_nodes) throw std::string("$Elements before $Nodes");
      if (m.version >= 4.0) read_v4_elements(c, m, phys);
      else read_v2_elements(c, m);
      have_elements = true;
    } else if (!tag.empty() && tag[0] == '$' && tag.compare(0, 4, "$end") != 0) {
      // any other section: skip to its end marker
      const std::string end = "$end" + tag.substr(1);
      while (c.token(t) && lower(t) != end) {
      }
    }
  }
  if (!have_format || !have_nodes || !have_elements)
    throw std::string("missing $MeshFormat, $Nodes or $Elements");
  for (const MshElem& e : m.elems) {
    const int nn = e.type == 2 ? 3 : 4;
    for (int k = 0; k < nn; k++)
      if (!m.node_at.count(e.node[k])) throw std::string("element refers to an unknown node");
  }
}

void put_node(const bem_msh& m, int64_t tag, double* out) {
  const int64_t i = m.node_at.at(tag);
  for (int d = 0; d < 3; d++) out[d] = m.xyz[3 * (size_t)i + d];
}

void copy_err(char* err, int64_t cap, const std::string& msg) {
  if (!err || cap <= 0) return;
  const size_t n = std::min<size_t>((size_t)cap - 1, msg.size());
  std::memcpy(err, msg.data(), n);
  err[n] = 0;
}

}  // namespace

extern "C" {

bem_status bem_msh_read(const char* path, bem_msh** out, char* err, int64_t errcap) {
  if (!out) return BEM_EINVAL;
  *out = nullptr;
  if (!path) {
    copy_err(err, errcap, "no path");
    return BEM_EINVAL;
  }
  std::FILE* f = std::fopen(path, "rb");
  if (!f) {
    copy_err(err, errcap, std::string("cannot open ") + path);
    return BEM_EINVAL;
  }
  std::string text;
  char buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
  std::fclose(f);
  bem_msh* m = new (std::nothrow) bem_msh;
  if (!m) return BEM_ENOMEM;
  try {
    parse(text, *m);
  } catch (const std::string& e) {
    copy_err(err, errcap, e);
    delete m;
    return BEM_EINVAL;
  } catch (const std::exception& e) {
    copy_err(err, errcap, e.what());
    delete m;
    return BEM_EINVAL;
  }
  // everything selected until bem_msh_select says otherwise
  for (size_t i = 0; i < m->elems.size(); i++)
    (m->elems[i].type == 2 ? m->sel_tri : m->sel_quad).push_back((int64_t)i);
  copy_err(err, errcap, "");
  *out = m;
  return BEM_OK;
}

void bem_msh_free(bem_msh* m) { delete m; }

int64_t bem_msh_num_physical(const bem_msh* m) { return m ? (int64_t)m->pname.size() : 0; }

bem_status bem_msh_physical(const bem_msh* m, int64_t i, int32_t* dim, int32_t* tag, char* name,
                            int64_t cap) {
  if (!m || i < 0 || i >= (int64_t)m->pname.size()) return BEM_EINVAL;
  if (dim) *dim = m->pdim[(size_t)i];
  if (tag) *tag = m->ptag[(size_t)i];
  copy_err(name, cap, m->pname[(size_t)i]);
  return BEM_OK;
}

bem_status bem_msh_select(bem_msh* m, const char* include, const char* exclude, int64_t* ntri,
                          int64_t* nquad) {
  if (!m) return BEM_EINVAL;
  std::vector<std::string> inc = split_list(include), exc = split_list(exclude);
  // "all" is dropped from the include list; the list then selects everything
  // (minus the excludes) only if nothing else is on it (:30-45)
  const auto is_all = [](const std::string& s) { return lower(s) == "all"; };
  inc.erase(std::remove_if(inc.begin(), inc.end(), is_all), inc.end());
  const bool include_all = inc.empty();
  const auto phys_of = [&](const std::string& name, int64_t& tag) {
    for (size_t k = 0; k < m->pname.size(); k++)
      if (lower(m->pname[k]) == lower(name)) {
        tag = m->ptag[k];
        return true;
      }
    return false;
  };
  std::vector<Interval> ginc, gexc;
  std::vector<int64_t> pinc, pexc;
  for (const std::string& t : inc) {
    Interval iv;
    bool empty = false;
    int64_t tag = 0;
    if (parse_range(t, iv, empty)) {
      if (!empty) ginc.push_back(iv);
    } else if (all_digits(t)) {
      const uint64_t v = std::strtoull(t.c_str(), nullptr, 10);
      ginc.push_back({v, v});
    } else if (phys_of(t, tag)) {
      pinc.push_back(tag);
    }
  }
  for (const std::string& t : exc) {
    Interval iv;
    bool empty = false;
    int64_t tag = 0;
    if (parse_range(t, iv, empty)) {
      if (!empty) gexc.push_back(iv);
    } else if (all_digits(t)) {
      const uint64_t v = std::strtoull(t.c_str(), nullptr, 10);
      gexc.push_back({v, v});
    } else if (include_all && phys_of(t, tag)) {
      // a name that is also on the include list is not excluded (:167-175)
      bool also_included = false;
      for (const std::string& u : inc) also_included |= lower(u) == lower(t);
      if (!also_included) pexc.push_back(tag);
    }
  }
  std::vector<Interval> gfilter;
  std::vector<int64_t> pfilter;
  if (include_all) {
    pfilter = pexc;
    gfilter = normalise(gexc);
  } else {
    pfilter = pinc;
    gfilter = difference(normalise(ginc), normalise(gexc));
  }
  m->sel_tri.clear();
  m->sel_quad.clear();
  for (size_t i = 0; i < m->elems.size(); i++) {
    const MshElem& e = m->elems[i];
    const bool in_p = std::find(pfilter.begin(), pfilter.end(), e.phys) != pfilter.end();
    const bool in_g = e.geom >= 0 && in_intervals((uint64_t)e.geom, gfilter);
    const bool keep = include_all ? !(in_p || in_g) : (in_p || in_g);
    if (keep) (e.type == 2 ? m->sel_tri : m->sel_quad).push_back((int64_t)i);
  }
  if (ntri) *ntri = (int64_t)m->sel_tri.size();
  if (nquad) *nquad = (int64_t)m->sel_quad.size();
  return BEM_OK;
}

bem_status bem_msh_elements(const bem_msh* m, double* tri, int32_t* tri_phys, int32_t* tri_geom,
                            double* quad, int32_t* quad_phys, int32_t* quad_geom) {
  if (!m) return BEM_EINVAL;
  for (size_t i = 0; i < m->sel_tri.size(); i++) {
    const MshElem& e = m->elems[(size_t)m->sel_tri[i]];
    if (tri)
      for (int k = 0; k < 3; k++) put_node(*m, e.node[k], tri + 9 * i + 3 * k);
    if (tri_phys) tri_phys[i] = (int32_t)e.phys;
    if (tri_geom) tri_geom[i] = (int32_t)e.geom;
  }
  for (size_t i = 0; i < m->sel_quad.size(); i++) {
    const MshElem& e = m->elems[(size_t)m->sel_quad[i]];
    if (quad)
      for (int k = 0; k < 4; k++) put_node(*m, e.node[k], quad + 12 * i + 3 * k);
    if (quad_phys) quad_phys[i] = (int32_t)e.phys;
    if (quad_geom) quad_geom[i] = (int32_t)e.geom;
  }
  return BEM_OK;
}

bem_status bem_quads_to_triangles(const double* quad, int64_t nq, double* tri) {
  if (nq < 0 || (nq > 0 && (!quad || !tri))) return BEM_EINVAL;
  for (int64_t i = 0; i < nq; i++) {
    const double* q = quad + 12 * i;
    double d1 = 0, d2 = 0;  // |n1 - n3|, |n2 - n4|
    for (int d = 0; d < 3; d++) {
      d1 += (q[d] - q[6 + d]) * (q[d] - q[6 + d]);
      d2 += (q[3 + d] - q[9 + d]) * (q[3 + d] - q[9 + d]);
    }
    // split along the shorter diagonal, node orders as the reference
    static const int a[2][3] = {{0, 1, 3}, {1, 2, 3}};  // d1 > d2
    static const int b[2][3] = {{3, 0, 2}, {0, 1, 2}};
    const int (*s)[3] = std::sqrt(d1) > std::sqrt(d2) ? a : b;
    for (int t = 0; t < 2; t++)
      for (int v = 0; v < 3; v++)
        for (int d = 0; d < 3; d++) tri[18 * i + 9 * t + 3 * v + d] = q[3 * s[t][v] + d];
  }
  return BEM_OK;
}

bem_status bem_refine_triangles(const double* tri, int64_t n, double edge_length, double* out,
                                int64_t cap, int64_t* nout, int64_t* parent) {
  if (n < 0 || (n > 0 && !tri) || !nout || !(edge_length > 0) || !std::isfinite(edge_length))
    return BEM_EINVAL;
  // ElementSection::refineTriangles / recursiveRefineTriangle
  // (SolvingScript/elementSection.cpp:688-800): a triangle whose longest edge
  // (indexOfMaxOfThree, :912, ties to the later edge) exceeds edge_length is
  // bisected at that edge's midpoint, node orders as the reference, and both
  // halves are refined in turn (depth first, first half first).
  const auto len = [](const double* a, const double* b) {
    return std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) +
                     (a[2] - b[2]) * (a[2] - b[2]));
  };
  const auto longest = [&](const double* t, double& e) {
    const double a = len(t, t + 3), b = len(t + 3, t + 6), c = len(t + 6, t);
    const int i = a > b ? (a > c ? 1 : 3) : (b > c ? 2 : 3);
    e = i == 1 ? a : (i == 2 ? b : c);
    return i;
  };
  int64_t count = 0;
  std::vector<std::array<double, 9>> stack;
  for (int64_t i = 0; i < n; i++) {
    stack.clear();
    std::array<double, 9> t0;
    for (int d = 0; d < 9; d++) t0[d] = tri[9 * i + d];
    stack.push_back(t0);
    while (!stack.empty()) {
      const std::array<double, 9> t = stack.back();
      stack.pop_back();
      double e = 0;
      const int k = longest(t.data(), e);
      if (!(e > edge_length)) {  // keep it
        if (out && count < cap) {
          for (int d = 0; d < 9; d++) out[9 * count + d] = t[d];
          if (parent) parent[count] = i;
        }
        count++;
        continue;
      }
      if (stack.size() > (size_t)1 << 20) return BEM_EINVAL;  // degenerate input
      const double* n1 = t.data();
      const double* n2 = t.data() + 3;
      const double* n3 = t.data() + 6;
      double m[3];
      const double* pa = k == 1 ? n1 : (k == 2 ? n2 : n3);
      const double* pb = k == 1 ? n2 : (k == 2 ? n3 : n1);
      for (int d = 0; d < 3; d++) m[d] = (pa[d] + pb[d]) / 2;
      std::array<double, 9> h1, h2;
      const auto put = [](std::array<double, 9>& h, const double* a, const double* b,
                          const double* c) {
        for (int d = 0; d < 3; d++) {
          h[d] = a[d];
          h[3 + d] = b[d];
          h[6 + d] = c[d];
        }
      };
      if (k == 1) {
        put(h1, n1, m, n3);
        put(h2, m, n2, n3);
      } else if (k == 2) {
        put(h1, n1, n2, m);
        put(h2, m, n3, n1);
      } else {
        put(h1, n1, n2, m);
        put(h2, m, n2, n3);
      }
      stack.push_back(h2);  // refined after h1
      stack.push_back(h1);
    }
  }
  *nout = count;
  return out && count > cap ? BEM_EINVAL : BEM_OK;
}

bem_status bem_wall_beta(int32_t imp_type, int32_t normalized, const double* value,
                         double medium_impedance, double* beta) {
  if (!value || !beta) return BEM_EINVAL;
  const std::complex<double> v(value[0], value[1]);
  std::complex<double> b;
  switch (imp_type) {
    case 0:  // Reflection: alpha = (1 - R) / (1 + R), R real
      b = (1.0 - v.real()) / (1.0 + v.real());
      break;
    case 1:  // Damping: alpha = d / (2 - d)
      b = v.real() / (2.0 - v.real());
      break;
    case 2:  // Impedance
      if (!normalized && medium_impedance == 0.0) return BEM_EINVAL;
      b = normalized ? 1.0 / v : medium_impedance / v;
      break;
    case 3:  // Admittance
      if (!normalized && medium_impedance == 0.0) return BEM_EINVAL;
      b = normalized ? v : medium_impedance * v;
      break;
    default:
      return BEM_EINVAL;
  }
  if (!std::isfinite(b.real()) || !std::isfinite(b.imag())) return BEM_ENONFINITE;
  beta[0] = b.real();
  beta[1] = b.imag();
  return BEM_OK;
}

}  // extern "C"
