// pm_deck.cu -- the reference's input decks: the mesh reader rdat_pm
// (Rdata.f:1-1037) with its block readers, the quadratic mesh generated from
// linear elements (mk_elconn_quad_v1, Adjacency.f:583-700; mk_coor_quad,
// Adjacency.f:907-955; mk_bound_quad / mk_forces_quad / mk_initial_quad,
// Rdata.f:2337-2544), the initial conditions of the end of the mesh macro
// (count_node_vertice, boundc, bound_nodalloads), and the macro program of
// Main.f (config, solver / pcg, gravity, nl / maxnlit, dt, setpnode, loop /
// next, solv, pnup, pnsf, stop) with a runner that drives the library's C ABI
// and writes the printnode history files (Pdata.f:733-790, names of
// Filenames.f:130-169).
//
// Words are read the way readmacro (Rdata.f:1945-2002) splits a line: runs
// of characters between blanks.  Blank lines and lines starting with "//" or
// "#" are skipped.  Blocks that the reference reads with list-directed input
// (elements, coordinates) take their numbers across line breaks.
//
// Older decks (the golden runs shipped with the reference) differ in four
// places, all accepted here: element codes 7 / 6 for hexa20 / tetra10 (now
// 17 / 15), "pcg maxit tol" for the solver, "maxnlit n" for the nonlinear
// loop (their runs accept the second nonlinear iteration, i.e. stop_crit 1),
// and loads of types 39-43 given inline as "type ncomp v1 .. vncomp" (a
// one-row table whose first column is the time) instead of a file name.
// Their runs did one solve per step and accepted it whatever maxnlit said, so
// "maxnlit n" reads as max(n, 2) nonlinear iterations with stop_crit 1.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/poromec_gb300.h"
#include "pm_loads.h"

namespace {

constexpr int kNdf = 4, kNtn = 6;

// hexa20edgeNod / tetra10edgeNod: (vertex, vertex, mid-side node), 1-based
const int kHexaEdges[12][3] = {{1, 2, 9},  {2, 3, 10}, {3, 4, 11}, {4, 1, 12},
                               {5, 6, 13}, {6, 7, 14}, {7, 8, 15}, {8, 5, 16},
                               {1, 5, 17}, {2, 6, 18}, {3, 7, 19}, {4, 8, 20}};
const int kTetraEdges[6][3] = {{1, 2, 5}, {1, 3, 6}, {1, 4, 7},
                               {2, 3, 8}, {3, 4, 9}, {4, 2, 10}};

enum OpKind { OP_SOLV, OP_PNUP, OP_PNSF, OP_LOOP, OP_NEXT, OP_DT, OP_NL, OP_SOLVER,
              OP_GRAVITY, OP_PGEO, OP_PRES, OP_STOP };

struct Settings {
  int solver = 11, precond = 2, maxit = 50000, maxnlit = 500, stop_crit = 2, nkrylov = 150;
  double solvtol = 1e-11, tol = 1e-4, dt = 1.0;
  double gravity[3] = {0.0, 0.0, -9.81};
};

struct Op {
  OpKind kind;
  Settings s;  // the settings after a settings op
  int n = 0;   // loop count
};

thread_local std::string g_err;  // message of the last failed pm_deck_* call of this thread

bool to_double(const std::string& t, double* v) {
  std::string u = t;
  for (char& c : u)
    if (c == 'd' || c == 'D') c = 'e';
  char* end = nullptr;
  *v = std::strtod(u.c_str(), &end);
  return end && *end == '\0' && !u.empty();
}

bool to_int(const std::string& t, long* v) {
  char* end = nullptr;
  *v = std::strtol(t.c_str(), &end, 10);
  return end && *end == '\0' && !t.empty();
}

// Fortran list-directed logical: an optional '.', then T or F (any case)
// decides; the rest of the word is ignored ("true", ".false.", "T").
bool fortran_logical(const std::string& t) {
  const size_t k = (!t.empty() && t[0] == '.') ? 1 : 0;
  return k < t.size() && (t[k] == 't' || t[k] == 'T');
}

std::vector<std::string> split(const std::string& line) {
  std::vector<std::string> w;
  std::string cur;
  for (char c : line) {
    if (c == ' ' || c == '\t' || c == '\r' || c == '\n') {
      if (!cur.empty()) w.push_back(cur);
      cur.clear();
    } else {
      cur += c;
    }
  }
  if (!cur.empty()) w.push_back(cur);
  return w;
}

std::string dir_of(const std::string& p) {
  const size_t k = p.find_last_of('/');
  return k == std::string::npos ? std::string(".") : p.substr(0, k);
}

std::string join(const std::string& dir, const std::string& name) {
  if (!name.empty() && name[0] == '/') return name;
  return dir + "/" + name;
}

// Lines of the deck with 'insert' files of the mesh macro spliced in.
class Reader {
  struct Src {
    std::vector<std::vector<std::string>> lines;
    std::vector<int> lineno;
    size_t pos = 0;
    std::string name;
  };
  std::vector<Src> st_;

 public:
  std::string err;
  bool push(const std::string& path) {
    std::ifstream in(path);
    if (!in) {
      err = "file " + path + " not found";
      return false;
    }
    Src s;
    s.name = path;
    std::string line;
    int ln = 0;
    while (std::getline(in, line)) {
      ++ln;
      auto w = split(line);
      if (w.empty() || w[0].rfind("//", 0) == 0 || w[0][0] == '#') continue;
      s.lines.push_back(std::move(w));
      s.lineno.push_back(ln);
    }
    st_.push_back(std::move(s));
    return true;
  }
  // the next line; an inserted file that ends returns to its parent
  bool next(std::vector<std::string>& w) {
    while (!st_.empty()) {
      Src& s = st_.back();
      if (s.pos < s.lines.size()) {
        w = s.lines[s.pos++];
        return true;
      }
      if (st_.size() == 1) return false;
      st_.pop_back();
    }
    return false;
  }
  void pop_insert() {
    if (st_.size() > 1) st_.pop_back();
  }
  std::string where() const {
    if (st_.empty()) return "";
    const Src& s = st_.back();
    const size_t k = s.pos ? s.pos - 1 : 0;
    return s.name + ":" + (k < s.lineno.size() ? std::to_string(s.lineno[k]) : "end");
  }
  // count numbers from the current line onwards (list-directed read)
  bool numbers(std::vector<std::string> first, size_t count, std::vector<std::string>& out) {
    out = std::move(first);
    std::vector<std::string> w;
    while (out.size() < count) {
      if (!next(w)) return false;
      out.insert(out.end(), w.begin(), w.end());
    }
    return true;
  }
};

}  // namespace

struct pm_deck_s {
  std::string path, dir;
  int nnode = 0, nnodev = 0, numel = 0, numat = 0, nen = 0, nenv = 0, ndf = 0, ndm = 0;
  bool elements_read = false, mk_quad = false, fstress0 = false, mesh_done = false;
  bool reord = true;  // reordf (Main.f:255): RCM node order unless config says false
  std::vector<int32_t> ix, ie, id, nload, eload, eloadp, fnno, load, print_nodes;
  std::vector<double> e, x, f, u0, tx0, fload;
  int nloads = 0, maxt = 1;
  Settings init;  // settings in force when the mesh macro ends
  Settings run0;  // settings in force at the first solv (at the end without one)
  bool have_run0 = false;
  std::vector<Op> prog;
  std::vector<std::string> node_macros, cell_macros;  // fields of the geometry file, read order
  int nunknown = 0;
};

namespace {

struct LoadTable {
  int type = 0, nparc = 1, nt = 1;
  std::map<std::pair<int, int>, double> v;  // (row l, column k) 1-based
};

bool fail(Reader& r, const std::string& what) {
  g_err = what + " (" + r.where() + ")";
  return false;
}

bool read_int(Reader& r, const std::string& t, long* v, const char* what) {
  if (!to_int(t, v)) return fail(r, std::string("expected an integer for ") + what + ", got '" +
                                        t + "'");
  return true;
}

bool read_real(Reader& r, const std::string& t, double* v, const char* what) {
  if (!to_double(t, v))
    return fail(r, std::string("expected a number for ") + what + ", got '" + t + "'");
  return true;
}

// parameters (Rdata.f:1863-1944): nnode numel numat maxno ndf dim, any order
bool read_parameters(Reader& r, pm_deck_s* d) {
  std::vector<std::string> w;
  if (!r.next(w)) return fail(r, "missing mesh parameters");
  std::map<std::string, long> kv;
  for (size_t i = 0; i + 1 < w.size(); i += 2) {
    long v;
    if (!read_int(r, w[i + 1], &v, w[i].c_str())) return false;
    kv[w[i]] = v;
  }
  for (const char* k : {"nnode", "numel", "numat", "maxno", "ndf", "dim"})
    if (!kv.count(k)) return fail(r, std::string("missing mesh parameter ") + k);
  d->nnodev = d->nnode = (int)kv["nnode"];
  d->numel = (int)kv["numel"];
  d->numat = (int)kv["numat"];
  d->nen = (int)kv["maxno"];
  d->ndf = (int)kv["ndf"];
  d->ndm = (int)kv["dim"];
  if (d->ndf != kNdf || d->ndm != 3 || !(d->nen == 20 || d->nen == 10))
    return fail(r, "the Biot path reads 3D poromechanical meshes (ndf 4, dim 3, maxno 20 or 10)");
  if (d->nnode <= 0 || d->numel <= 0 || d->numat <= 0) return fail(r, "empty mesh");
  d->nenv = d->nen == 20 ? 8 : 4;
  d->ix.assign((size_t)(d->nen + 1) * d->numel, 0);
  d->ie.assign(d->numat, 0);
  d->e.assign((size_t)PM_PROP * d->numat, 0.0);
  d->x.assign((size_t)3 * d->nnode, 0.0);
  d->eload.assign((size_t)7 * d->numel, 0);
  d->eloadp.assign((size_t)7 * d->numel, 0);
  return true;
}

void node_arrays(pm_deck_s* d) {
  const size_t n = d->nnode;
  d->id.assign(kNdf * n, 0);
  d->nload.assign(kNdf * n, 0);
  d->f.assign(kNdf * n, 0.0);
  d->u0.assign(kNdf * n, 0.0);
  d->tx0.assign(kNtn * n, 0.0);
}

// mate (Rdata.f:1132-1183): "ma code e1 e2 ..." until 'end'
bool read_materials(Reader& r, pm_deck_s* d) {
  std::vector<std::string> w;
  while (r.next(w) && w[0] != "end") {
    long ma, code;
    if (!read_int(r, w[0], &ma, "material") || w.size() < 2 ||
        !read_int(r, w[1], &code, "element code"))
      return false;
    if (ma < 1 || ma > d->numat) return fail(r, "material number out of range");
    if (code == 7) code = 17;  // old element codes of the golden decks
    if (code == 6) code = 15;
    d->ie[ma - 1] = (int)code;
    if (w.size() - 2 > (size_t)PM_PROP) return fail(r, "too many material properties");
    for (size_t k = 2; k < w.size(); ++k)
      if (!read_real(r, w[k], &d->e[(size_t)PM_PROP * (ma - 1) + k - 2], "material property"))
        return false;
  }
  return true;
}

// file_prop (Rdata.f:2683-2928) for the elastic Biot elements: a file per
// material with its element code and properties as "name value" pairs
bool read_fmaterials(Reader& r, pm_deck_s* d) {
  static const char* names[] = {"young", "poisson", "permeability", "biotmodulus",
                                "biotcoefficient", "density", "fluiddensity", "porosity"};
  std::vector<std::string> w;
  while (r.next(w) && w[0] != "end") {
    long ma;
    if (!read_int(r, w[0], &ma, "material") || w.size() < 2) return false;
    if (ma < 1 || ma > d->numat) return fail(r, "material number out of range");
    Reader fr;
    if (!fr.push(join(d->dir, w[1]))) return fail(r, fr.err);
    std::vector<std::string> v;
    while (fr.next(v) && v[0] != "end") {
      if (v.size() < 2) continue;
      if (v[0] == "elmt" || v[0] == "element") {
        long code;
        if (!read_int(fr, v[1], &code, "element code")) return false;
        d->ie[ma - 1] = (int)(code == 7 ? 17 : code == 6 ? 15 : code);
        continue;
      }
      for (int k = 0; k < 8; ++k)
        if (v[0] == names[k] &&
            !read_real(fr, v[1], &d->e[(size_t)PM_PROP * (ma - 1) + k], names[k]))
          return false;
    }
  }
  return true;
}

// mk_elconn_quad_v1 (Adjacency.f:583-700): mid-side nodes numbered after
// the vertices, element by element, shared with the elements on the edge
bool make_quadratic(pm_deck_s* d) {
  const int nen = d->nen, nenv = d->nenv, numel = d->numel, nnodev = d->nnodev;
  const int ne = nen == 20 ? 12 : 6;
  const int(*edges)[3] = nen == 20 ? kHexaEdges : kTetraEdges;
  std::vector<std::vector<int>> incid(nnodev + 1);
  for (int el = 0; el < numel; ++el)
    for (int k = 0; k < nenv; ++k) {
      const int v = d->ix[(size_t)(nen + 1) * el + k];
      if (v < 1 || v > nnodev) return false;
      incid[v].push_back(el);
    }
  int nno = nnodev;
  auto IX = [&](int el, int k) -> int32_t& { return d->ix[(size_t)(nen + 1) * el + k]; };
  for (int el = 0; el < numel; ++el) {
    for (int j = nenv; j < nen; ++j)
      if (IX(el, j) == 0) IX(el, j) = ++nno;
    for (int a = 0; a < ne; ++a) {
      const int no1 = IX(el, edges[a][0] - 1), no2 = IX(el, edges[a][1] - 1);
      const int no3 = IX(el, edges[a][2] - 1);
      for (int nel : incid[no1]) {
        if (nel == el) continue;
        for (int b = 0; b < ne; ++b) {
          const int v1 = IX(nel, edges[b][0] - 1), v2 = IX(nel, edges[b][1] - 1);
          if (((no1 == v1 && no2 == v2) || (no1 == v2 && no2 == v1)) &&
              IX(nel, edges[b][2] - 1) == 0)
            IX(nel, edges[b][2] - 1) = no3;
        }
      }
    }
  }
  d->nnode = nno;
  // mk_coor_quad: mid-side coordinates at the edge midpoints
  std::vector<double> x((size_t)3 * nno, 0.0);
  std::copy(d->x.begin(), d->x.begin() + (size_t)3 * nnodev, x.begin());
  for (int el = 0; el < numel; ++el)
    for (int a = 0; a < ne; ++a) {
      const int no1 = IX(el, edges[a][0] - 1), no2 = IX(el, edges[a][1] - 1);
      const int no3 = IX(el, edges[a][2] - 1);
      for (int k = 0; k < 3; ++k)
        x[(size_t)3 * (no3 - 1) + k] =
            0.5 * (x[(size_t)3 * (no1 - 1) + k] + x[(size_t)3 * (no2 - 1) + k]);
    }
  d->x.swap(x);
  return true;
}

// elconn (Rdata.f:1038-1089) of linear or quadratic elements
bool read_elements(Reader& r, pm_deck_s* d, int nv_in) {
  if (d->elements_read) return fail(r, "elements given twice");
  std::vector<std::string> w, t;
  for (int j = 0; j < d->numel; ++j) {
    if (!r.next(w) || !r.numbers(w, nv_in + 2, t)) return fail(r, "missing element lines");
    long k;
    if (!read_int(r, t[0], &k, "element")) return false;
    if (k < 1 || k > d->numel) return fail(r, "element number out of range");
    for (int m = 0; m <= nv_in; ++m) {
      long v;
      if (!read_int(r, t[1 + m], &v, "element node")) return false;
      const int slot = m < nv_in ? m : d->nen;
      d->ix[(size_t)(d->nen + 1) * (k - 1) + slot] = (int32_t)v;
    }
  }
  if (!r.next(w) || w[0] != "end") return fail(r, "element block without 'end'");
  d->elements_read = true;
  if (nv_in == d->nenv) {
    d->mk_quad = true;
    if (!make_quadratic(d)) return fail(r, "vertex node id out of range");
  }
  node_arrays(d);
  return true;
}

// coord (Rdata.f:1090-1131): nnode lines of "k x y z"
bool read_coordinates(Reader& r, pm_deck_s* d) {
  std::vector<std::string> w, t;
  const int n = d->elements_read && d->mk_quad ? d->nnodev : d->nnode;
  for (int j = 0; j < n; ++j) {
    if (!r.next(w) || !r.numbers(w, 4, t)) return fail(r, "missing coordinate lines");
    long k;
    if (!read_int(r, t[0], &k, "node")) return false;
    if (k < 1 || k > n) return fail(r, "node number out of range");
    for (int m = 0; m < 3; ++m)
      if (!read_real(r, t[1 + m], &d->x[(size_t)3 * (k - 1) + m], "coordinate")) return false;
  }
  if (!r.next(w) || w[0] != "end") return fail(r, "coordinate block without 'end'");
  if (d->elements_read && d->mk_quad) {
    // coordinates after the elements: mid-side nodes at the edge midpoints
    const int nen = d->nen, ne = nen == 20 ? 12 : 6;
    const int(*edges)[3] = nen == 20 ? kHexaEdges : kTetraEdges;
    for (int el = 0; el < d->numel; ++el)
      for (int a = 0; a < ne; ++a) {
        const int32_t* nd = &d->ix[(size_t)(nen + 1) * el];
        const int no1 = nd[edges[a][0] - 1], no2 = nd[edges[a][1] - 1];
        const int no3 = nd[edges[a][2] - 1];
        for (int k = 0; k < 3; ++k)
          d->x[(size_t)3 * (no3 - 1) + k] =
              0.5 * (d->x[(size_t)3 * (no1 - 1) + k] + d->x[(size_t)3 * (no2 - 1) + k]);
      }
  }
  return true;
}

// bound (Rdata.f:1408-1456): "j v1 v2 .. (up to width)" until 'end'
bool read_int_rows(Reader& r, std::vector<int32_t>& a, int width, int nmax, const char* what) {
  std::vector<std::string> w;
  while (r.next(w) && w[0] != "end") {
    long j;
    if (!read_int(r, w[0], &j, what)) return false;
    if (j < 1 || j > nmax) return fail(r, std::string(what) + " number out of range");
    if ((int)w.size() - 1 > width) return fail(r, std::string("too many values for ") + what);
    for (size_t i = 1; i < w.size(); ++i) {
      long v;
      if (!read_int(r, w[i], &v, what)) return false;
      a[(size_t)width * (j - 1) + i - 1] = (int32_t)v;
    }
  }
  return true;
}

// forces / init_poro_mec (Rdata.f:1236-1300): "k v(n1) .. v(n2)" until 'end'
bool read_real_rows(Reader& r, std::vector<double>& a, int width, int n1, int n2, int nmax,
                    const char* what) {
  std::vector<std::string> w;
  while (r.next(w) && w[0] != "end") {
    long k;
    if (!read_int(r, w[0], &k, what)) return false;
    if (k < 1 || k > nmax) return fail(r, std::string(what) + " node out of range");
    if ((int)w.size() < 2 + n2 - n1) return fail(r, std::string("missing values for ") + what);
    for (int j = n1; j <= n2; ++j)
      if (!read_real(r, w[1 + j - n1], &a[(size_t)width * (k - 1) + j - 1], what)) return false;
  }
  return true;
}

// mk_bound_quad / mk_forces_quad / mk_initial_quad (Rdata.f:2337-2544)
template <typename F>
void for_edges(const pm_deck_s* d, F fn) {
  const int nen = d->nen, ne = nen == 20 ? 12 : 6;
  const int(*edges)[3] = nen == 20 ? kHexaEdges : kTetraEdges;
  for (int el = 0; el < d->numel; ++el)
    for (int a = 0; a < ne; ++a) {
      const int32_t* nd = &d->ix[(size_t)(nen + 1) * el];
      fn(nd[edges[a][0] - 1] - 1, nd[edges[a][1] - 1] - 1, nd[edges[a][2] - 1] - 1);
    }
}

// rload (Rdata.f:1487-1671)
bool read_loads(Reader& r, pm_deck_s* d, std::map<int, LoadTable>& tabs) {
  std::vector<std::string> w;
  while (r.next(w) && w[0] != "end") {
    long i, ty;
    if (!read_int(r, w[0], &i, "load") || w.size() < 2 || !read_int(r, w[1], &ty, "load type"))
      return false;
    if (i < 1 || i > 200) return fail(r, "load number out of range (1..200)");
    LoadTable T;
    T.type = (int)ty;
    size_t p = 2;
    auto num = [&](double* v) -> bool {
      if (p >= w.size()) {
        std::vector<std::string> more;
        if (!r.next(more)) return fail(r, "load values missing");
        w.insert(w.end(), more.begin(), more.end());
      }
      return read_real(r, w[p++], v, "load value");
    };
    auto cnt = [&](int* v) -> bool {
      double x;
      if (!num(&x)) return false;
      *v = (int)x;
      return true;
    };
    double v;
    if (ty == 1) {
      if (!num(&v)) return false;
      T.v[{1, 1}] = v;
    } else if (ty == 2 || ty == 3) {
      if (!num(&v)) return false;
      T.v[{1, 1}] = v;
      if (!num(&v)) return false;
      T.v[{2, 1}] = v;
    } else if (ty == 6) {
      if (!cnt(&T.nparc)) return false;
      for (int k = 1; k <= T.nparc; ++k)
        for (int l = 1; l <= 3; ++l) {
          if (!num(&v)) return false;
          T.v[{l, k}] = v;
        }
    } else if (ty >= 39 && ty <= 43) {
      long nc;
      if (p < w.size() && to_int(w[p], &nc)) {
        // older decks: "type ncomp v1 .. vncomp", a one-row table after the time column
        ++p;
        T.nparc = (int)nc + 1;
        T.nt = 1;
        T.v[{1, 1}] = 0.0;
        for (int k = 2; k <= T.nparc; ++k) {
          if (!num(&v)) return false;
          T.v[{1, k}] = v;
        }
      } else {
        if (p >= w.size()) return fail(r, "load file name missing");
        Reader fr;
        if (!fr.push(join(d->dir, w[p]))) return fail(r, fr.err);
        std::vector<std::string> fw, vals;
        if (!fr.next(fw)) return fail(fr, "empty load file");
        long np, nt;
        if (fw.size() < 2 || !read_int(fr, fw[0], &np, "load columns") ||
            !read_int(fr, fw[1], &nt, "load rows"))
          return false;
        T.nparc = (int)np;
        T.nt = (int)nt;
        for (int l = 1; l <= T.nt; ++l) {
          if (!fr.next(fw) || !fr.numbers(fw, T.nparc, vals)) return fail(fr, "load rows missing");
          for (int k = 1; k <= T.nparc; ++k) {
            if (!read_real(fr, vals[k - 1], &v, "load value")) return false;
            T.v[{l, k}] = v;
          }
        }
      }
    } else {
      return fail(r, "load type " + std::to_string(ty) + " is not one of the Biot path's");
    }
    if (T.nparc > PM_NFLOAD) return fail(r, "load with more columns than PM_NFLOAD");
    tabs[(int)i] = T;
  }
  return true;
}

void finish_loads(pm_deck_s* d, const std::map<int, LoadTable>& tabs) {
  d->nloads = tabs.empty() ? 0 : tabs.rbegin()->first;
  int maxt = 1;
  for (const auto& kv : tabs)
    for (const auto& e : kv.second.v) maxt = std::max(maxt, e.first.first);
  d->maxt = maxt;
  d->load.assign((size_t)3 * d->nloads, 0);
  d->fload.assign((size_t)maxt * PM_NFLOAD * d->nloads, 0.0);
  for (const auto& kv : tabs) {
    const int i = kv.first - 1;
    d->load[3 * i] = kv.second.type;
    d->load[3 * i + 1] = kv.second.nparc;
    d->load[3 * i + 2] = kv.second.nt;
    for (const auto& e : kv.second.v)
      d->fload[(size_t)maxt * PM_NFLOAD * i + (size_t)maxt * (e.first.second - 1) +
               e.first.first - 1] = e.second;
  }
}

// hydrostatic (init_hydrostatic_pres, Rdata.f:1301-1349) and hydrostress
// (init_hydrostatic_stress, Rdata.f:1350-1407): a file of parameters
bool read_hydro(Reader& r, pm_deck_s* d, const std::vector<std::string>& w, bool stress,
                const Settings& s) {
  if (w.size() < 2) return fail(r, "hydrostatic file name missing");
  Reader fr;
  if (!fr.push(join(d->dir, w[1]))) return fail(r, fr.err);
  std::vector<std::string> fw, vals;
  if (!fr.next(fw) || !fr.numbers(fw, stress ? 5 : 4, vals)) return fail(fr, "values missing");
  double p[5];
  for (int k = 0; k < (stress ? 5 : 4); ++k)
    if (!read_real(fr, vals[k], &p[k], "hydrostatic parameter")) return false;
  const double gmod = std::sqrt(s.gravity[0] * s.gravity[0] + s.gravity[1] * s.gravity[1] +
                                s.gravity[2] * s.gravity[2]);
  for (int i = 0; i < d->nnode; ++i) {
    const double z = d->x[(size_t)3 * i + 2];
    if (!stress) {
      d->u0[(size_t)kNdf * i + 3] = (p[1] + p[0] * gmod * (p[2] - z)) * p[3];
    } else {
      double* t = &d->tx0[(size_t)kNtn * i];
      t[2] = (p[1] + p[0] * gmod * (p[2] - z)) * p[4];
      t[0] = p[3] * t[2];
      t[1] = p[3] * t[2];
      t[3] = t[4] = t[5] = 0.0;
    }
  }
  if (stress) d->fstress0 = true;
  return true;
}

// the end of the mesh macro (Rdata.f:930-1037)
bool finish_mesh(Reader& r, pm_deck_s* d) {
  if (!d->elements_read) return fail(r, "mesh without elements");
  for (int k = 0; k < d->numat; ++k)
    if (!((d->nen == 20 && d->ie[k] == 17) || (d->nen == 10 && d->ie[k] == 15)))
      return fail(r, "material " + std::to_string(k + 1) +
                         " has no elastic Biot element type (17 hexa20, 15 tetra10)");
  // count_node_vertice: vertex nodes
  d->fnno.assign(d->nnode, 0);
  int nv = 0;
  for (int el = 0; el < d->numel; ++el)
    for (int k = 0; k < d->nenv; ++k) {
      const int v = d->ix[(size_t)(d->nen + 1) * el + k];
      if (v < 1 || v > d->nnode) return fail(r, "element node out of range");
      if (!d->fnno[v - 1]) ++nv;
      d->fnno[v - 1] = 1;
    }
  if (!d->mk_quad) d->nnodev = nv;
  // boundc: restrained dofs take their prescribed values
  for (size_t q = 0; q < d->u0.size(); ++q)
    if (d->id[q] > 0) d->u0[q] = d->f[q];
  // bound_nodalloads: time loads of restrained dofs at t = 0
  const double gmod = std::sqrt(d->init.gravity[0] * d->init.gravity[0] +
                                d->init.gravity[1] * d->init.gravity[1] +
                                d->init.gravity[2] * d->init.gravity[2]);
  for (int i = 0; i < d->nnode; ++i)
    for (int j = 0; j < kNdf; ++j) {
      const size_t q = (size_t)kNdf * i + j;
      const int nc = d->nload[q];
      if (nc > 0 && d->id[q] == 1) {
        if (nc > d->nloads) return fail(r, "nodal load id without a load");
        d->u0[q] = pm::nodal_load(d->load.data(), d->fload.data(), d->maxt, nc, 0.0,
                                  &d->x[(size_t)3 * i], d->u0[q], gmod);
      }
    }
  d->mesh_done = true;
  return true;
}

// rdat_pm macro loop (Rdata.f:355-1037)
bool read_mesh(Reader& r, pm_deck_s* d, const Settings& s) {
  if (!read_parameters(r, d)) return false;
  std::map<int, LoadTable> tabs;
  std::vector<std::string> w;
  auto need_el = [&](const char* what) {
    if (!d->elements_read)
      return fail(r, std::string("macro ") + what + " before the elements (Unread Elements)");
    return true;
  };
  while (r.next(w)) {
    const std::string& m = w[0];
    for (const char* k : {"constrainpmec", "constraindisp", "nodalforces", "nodalloads",
                          "initialpres", "initialstress"})
      if (m == k) d->node_macros.push_back(m);
    for (const char* k : {"elmtloads", "elmtpresloads"})
      if (m == k) d->cell_macros.push_back(m);
    if (m == "end") {
      finish_loads(d, tabs);
      return finish_mesh(r, d);
    } else if (m == "materials") {
      if (!read_materials(r, d)) return false;
    } else if (m == "fmaterials") {
      if (!read_fmaterials(r, d)) return false;
    } else if (m == "hexa8" || m == "tetra4" || m == "hexa20" || m == "tetra10") {
      const int nv = m == "hexa8" ? 8 : m == "tetra4" ? 4 : m == "hexa20" ? 20 : 10;
      if ((d->nen == 20) != (nv == 8 || nv == 20))
        return fail(r, "element block " + m + " does not match maxno");
      if (!read_elements(r, d, nv)) return false;
    } else if (m == "coordinates") {
      if (!read_coordinates(r, d)) return false;
    } else if (m == "constrainpmec" || m == "constraindisp") {
      if (!need_el(m.c_str()) || !read_int_rows(r, d->id, kNdf, d->nnodev, "restraint"))
        return false;
      if (d->mk_quad)
        for_edges(d, [&](int a, int b, int c) {
          for (int k = 0; k < kNdf - 1; ++k)
            if (d->id[kNdf * a + k] == 1 && d->id[kNdf * b + k] == 1) d->id[kNdf * c + k] = 1;
        });
    } else if (m == "nodalforces") {
      if (!need_el(m.c_str()) ||
          !read_real_rows(r, d->f, kNdf, 1, kNdf, d->nnodev, "nodal force"))
        return false;
      if (d->mk_quad)
        for_edges(d, [&](int a, int b, int c) {
          for (int k = 0; k < kNdf - 1; ++k)
            if (d->id[kNdf * a + k] == 1 && d->id[kNdf * b + k] == 1)
              d->f[kNdf * c + k] = 0.5 * (d->f[kNdf * a + k] + d->f[kNdf * b + k]);
        });
    } else if (m == "elmtloads") {
      if (!read_int_rows(r, d->eload, 7, d->numel, "element load")) return false;
    } else if (m == "elmtpresloads") {
      if (!read_int_rows(r, d->eloadp, 7, d->numel, "element pressure load")) return false;
    } else if (m == "nodalloads") {
      if (!need_el(m.c_str()) || !read_int_rows(r, d->nload, kNdf, d->nnodev, "nodal load"))
        return false;
    } else if (m == "loads") {
      if (!read_loads(r, d, tabs)) return false;
    } else if (m == "initialpres") {
      if (!need_el(m.c_str()) ||
          !read_real_rows(r, d->u0, kNdf, kNdf, kNdf, d->nnodev, "initial pressure"))
        return false;
    } else if (m == "initialdisp") {
      if (!need_el(m.c_str()) ||
          !read_real_rows(r, d->u0, kNdf, 1, kNdf - 1, d->nnode, "initial displacement"))
        return false;
    } else if (m == "initialstress") {
      if (!need_el(m.c_str()) ||
          !read_real_rows(r, d->tx0, kNtn, 1, kNtn, d->nnodev, "initial stress"))
        return false;
      if (d->mk_quad)
        for_edges(d, [&](int a, int b, int c) {
          for (int k = 0; k < kNtn; ++k)
            d->tx0[kNtn * c + k] = 0.5 * (d->tx0[kNtn * a + k] + d->tx0[kNtn * b + k]);
        });
      d->fstress0 = true;
    } else if (m == "hydrostatic" || m == "hydrostress") {
      if (!need_el(m.c_str()) || !read_hydro(r, d, w, m == "hydrostress", s)) return false;
    } else if (m == "insert") {
      if (w.size() < 2) return fail(r, "insert without a file name");
      if (!r.push(join(d->dir, w[1]))) return fail(r, r.err);
    } else if (m == "return") {
      r.pop_insert();
    } else {
      ++d->nunknown;
    }
  }
  return fail(r, "mesh macro without 'end'");
}

// read_solver_config_pm (Rdata.f:3141-3382): a file of "key value" pairs
bool read_solver_file(Reader& r, pm_deck_s* d, const std::string& name, Settings& s) {
  Reader fr;
  if (!fr.push(join(d->dir, name))) return fail(r, fr.err);
  std::vector<std::string> w;
  static const std::map<std::string, int> solvers = {
      {"cg", 1}, {"sqmr", 11}, {"minres", 7}, {"gmres", 2}};
  static const std::map<std::string, int> preconds = {
      {"none", 1}, {"diag", 2}, {"ildlt", 3}, {"illt", 4}, {"diagm", 5}, {"bdiag", 6},
      {"diags", 7}};
  while (fr.next(w) && w[0] != "end") {
    if (w.size() < 2) continue;
    long iv;
    double dv;
    if (w[0] == "name") {
      auto it = solvers.find(w[1]);
      if (it == solvers.end())
        return fail(fr, "solver " + w[1] + " is not on the Biot path (cg, minres, sqmr, gmres)");
      s.solver = it->second;
    } else if (w[0] == "it") {
      if (!read_int(fr, w[1], &iv, "it")) return false;
      s.maxit = (int)iv;
    } else if (w[0] == "tol") {
      if (!read_real(fr, w[1], &dv, "tol")) return false;
      s.solvtol = dv == 0.0 ? std::ldexp(1.0, -53) : dv;
    } else if (w[0] == "precond") {
      auto it = preconds.find(w[1]);
      if (it == preconds.end() || !(it->second == 2 || it->second == 5))
        return fail(fr, "preconditioner " + w[1] + " is not on the Biot path (diag, diagm)");
      s.precond = it->second;
    } else if (w[0] == "nkrylov" || w[0] == "nKrylov") {
      if (!read_int(fr, w[1], &iv, "nkrylov")) return false;
      s.nkrylov = (int)iv;
    }
  }
  return true;
}

bool parse(Reader& r, pm_deck_s* d) {
  Settings s;
  std::vector<std::string> w;
  auto settings_op = [&](OpKind k) {
    Op op;
    op.kind = k;
    op.s = s;
    d->prog.push_back(op);
  };
  int depth = 0;
  while (r.next(w)) {
    const std::string& m = w[0];
    if (m == "mesh") {
      if (d->mesh_done) return fail(r, "second mesh macro");
      d->init = s;
      if (!read_mesh(r, d, s)) return false;
      d->init = s;
    } else if (m == "config") {
      // read_config (Rdata.f:2929-3110): "key value" pairs up to 'end', inline
      // in the older decks, in a named file in the current syntax; only
      // reord changes what the library computes (RCM node order, on by
      // default as reordf in Main.f:255)
      Reader cf;
      Reader* src = &r;
      if (w.size() >= 2) {
        if (!cf.push(join(d->dir, w[1]))) return fail(r, cf.err);
        src = &cf;
      }
      while (src->next(w) && w[0] != "end")
        for (size_t k = 0; k + 1 < w.size(); k += 2)
          if (w[k] == "reord") d->reord = fortran_logical(w[k + 1]);
    } else if (m == "pcg") {  // older decks: "pcg maxit tol"
      long it;
      double tol;
      if (w.size() < 3 || !read_int(r, w[1], &it, "pcg maxit") ||
          !read_real(r, w[2], &tol, "pcg tol"))
        return false;
      s.solver = 1;
      s.maxit = (int)it;
      s.solvtol = tol == 0.0 ? std::ldexp(1.0, -53) : tol;
      settings_op(OP_SOLVER);
    } else if (m == "solver") {
      if (w.size() < 2) return fail(r, "solver file missing");
      if (!read_solver_file(r, d, w[1], s)) return false;
      settings_op(OP_SOLVER);
    } else if (m == "gravity") {
      double g[3];
      if (w.size() >= 4 && to_double(w[1], &g[0])) {  // older decks: inline components
        for (int k = 0; k < 3; ++k)
          if (!read_real(r, w[1 + k], &g[k], "gravity")) return false;
      } else {
        // read_gravity (Rdata.f:3543-3600): a file with gx gy gz |g|
        if (w.size() < 2) return fail(r, "gravity file missing");
        Reader fr;
        if (!fr.push(join(d->dir, w[1]))) return fail(r, fr.err);
        std::vector<std::string> fw, vals;
        if (!fr.next(fw) || !fr.numbers(fw, 3, vals)) return fail(fr, "gravity values missing");
        for (int k = 0; k < 3; ++k)
          if (!read_real(fr, vals[k], &g[k], "gravity")) return false;
      }
      for (int k = 0; k < 3; ++k) s.gravity[k] = g[k];
      settings_op(OP_GRAVITY);
    } else if (m == "maxnlit") {
      // older decks: their runs did one solve per step and accepted it (also
      // with maxnlit 1), i.e. the second iteration's check of stop_crit 1
      long n;
      if (w.size() < 2 || !read_int(r, w[1], &n, "maxnlit")) return false;
      s.maxnlit = std::max(2, (int)n);
      s.stop_crit = 1;
      settings_op(OP_NL);
    } else if (m == "nl") {
      long n, sc;
      double tol;
      if (w.size() < 4 || !read_int(r, w[1], &n, "nl maxnlit") ||
          !read_real(r, w[2], &tol, "nl tol") || !read_int(r, w[3], &sc, "nl stop_crit"))
        return false;
      s.maxnlit = (int)n;
      s.tol = tol;
      s.stop_crit = (int)sc;
      settings_op(OP_NL);
    } else if (m == "dt") {
      if (w.size() < 2 || !read_real(r, w[1], &s.dt, "dt")) return false;
      settings_op(OP_DT);
    } else if (m == "setpnode") {
      if (w.size() < 2) return fail(r, "setpnode without a file");
      Reader fr;
      if (!fr.push(join(d->dir, w[1]))) return fail(r, fr.err);
      std::vector<std::string> fw, vals;
      long n;
      if (!fr.next(fw) || !read_int(fr, fw[0], &n, "number of nodes")) return false;
      fw.erase(fw.begin());
      if (fw.empty() && n > 0 && !fr.next(fw)) return fail(fr, "node ids missing");
      if (n > 0 && !fr.numbers(fw, (size_t)n, vals)) return fail(fr, "node ids missing");
      d->print_nodes.clear();
      for (long k = 0; k < n; ++k) {
        long v;
        if (!read_int(fr, vals[k], &v, "node")) return false;
        d->print_nodes.push_back((int32_t)v);
      }
    } else if (m == "loop") {
      long n;
      if (w.size() < 2 || !read_int(r, w[1], &n, "loop count")) return false;
      Op op;
      op.kind = OP_LOOP;
      op.n = (int)n;
      d->prog.push_back(op);
      ++depth;
    } else if (m == "next") {
      if (depth == 0) return fail(r, "'next' without 'loop'");
      --depth;
      d->prog.push_back(Op{OP_NEXT});
    } else if (m == "solv") {
      if (!d->have_run0) {
        d->run0 = s;
        d->have_run0 = true;
      }
      d->prog.push_back(Op{OP_SOLV});
    } else if (m == "pnup") {
      d->prog.push_back(Op{OP_PNUP});
    } else if (m == "pnsf") {
      d->prog.push_back(Op{OP_PNSF});
    } else if (m == "pgeo") {
      d->prog.push_back(Op{OP_PGEO});
    } else if (m == "pres") {
      d->prog.push_back(Op{OP_PRES});
    } else if (m == "stop") {
      d->prog.push_back(Op{OP_STOP});
      break;
    } else {
      ++d->nunknown;
    }
  }
  if (!d->have_run0) d->run0 = s;
  if (depth != 0) return fail(r, "'loop' without 'next'");
  if (!d->mesh_done) return fail(r, "deck without a mesh macro");
  return true;
}

// printnode (Pdata.f:733-790): "(i9,10e18.10)" rows, or the column layout of
// the golden runs' files (i9, f30.6, f30.10 ...)
std::string fortran_e18_10(double v) {
  if (v == 0.0 || !std::isfinite(v)) {
    char b[64];
    if (v == 0.0)
      std::snprintf(b, sizeof b, "%18s", "0.0000000000E+00");
    else
      std::snprintf(b, sizeof b, "%18s",
                    std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity"));
    return b;
  }
  char m[64];
  std::snprintf(m, sizeof m, "%.9E", v);  // d.ddddddddd E+xx, 10 significant digits
  const char* p = m;
  const bool neg = *p == '-';
  if (neg) ++p;
  std::string digits;
  for (; *p && *p != 'E'; ++p)
    if (*p != '.') digits += *p;
  const int ex = std::atoi(p + 1) + 1;
  char b[64];
  if (std::abs(ex) <= 99)
    std::snprintf(b, sizeof b, "%s0.%sE%c%02d", neg ? "-" : "", digits.c_str(),
                  ex < 0 ? '-' : '+', std::abs(ex));
  else
    std::snprintf(b, sizeof b, "%s0.%s%c%03d", neg ? "-" : "", digits.c_str(),
                  ex < 0 ? '-' : '+', std::abs(ex));
  char o[64];
  std::snprintf(o, sizeof o, "%18s", b);
  return o;
}

struct Printer {
  std::string prefix;
  int format;  // 0 printnode (current), 1 the golden runs' layout
  std::map<std::string, bool> opened;
  int print(const std::string& tag, const std::string& name, int node, int istep, double t,
            const double* v, int n) {
    const std::string fn = prefix + "_" + tag + "_node_" + std::to_string(node) + ".txt";
    const bool first = !opened[fn];
    FILE* f = std::fopen(fn.c_str(), first ? "w" : "a");
    if (!f) {
      g_err = "cannot write " + fn;
      return PM_E_ARG;
    }
    if (first) std::fprintf(f, "# Variacao %s no tempo no ponto%9d\n", name.c_str(), node);
    opened[fn] = true;
    std::fprintf(f, "%9d", istep);
    if (format == 1) {
      std::fprintf(f, "%30.6f", t);
      for (int k = 0; k < n; ++k) std::fprintf(f, "%30.10f", v[k]);
    } else {
      std::fputs(fortran_e18_10(t).c_str(), f);
      for (int k = 0; k < n; ++k) std::fputs(fortran_e18_10(v[k]).c_str(), f);
    }
    std::fputc('\n', f);
    std::fclose(f);
    return PM_OK;
  }
};

// ---- legacy ASCII VTK (Vtk.f, Write_vtk.f) ----------------------------------
// Fortran Ew.d / Ew.dEe edit descriptors: 0.d1..dd mantissa, the exponent
// with e digits (2 by default, the form without 'E' past 99).
std::string fortran_e(double v, int w, int dd, int edig) {
  char b[64];
  if (!std::isfinite(v)) {
    std::snprintf(b, sizeof b, "%*s", w, std::isnan(v) ? "NaN" : v > 0 ? "Infinity" : "-Infinity");
    return b;
  }
  int ex = 0;
  std::string digits(dd, '0');
  bool neg = std::signbit(v) && v != 0.0;
  if (v != 0.0) {
    char m[64];
    std::snprintf(m, sizeof m, "%.*E", dd - 1, v);
    const char* p = m;
    if (*p == '-') ++p;
    digits.clear();
    for (; *p && *p != 'E'; ++p)
      if (*p != '.') digits += *p;
    ex = std::atoi(p + 1) + 1;
  }
  char e[16];
  if (std::abs(ex) < (edig == 2 ? 100 : 1000))
    std::snprintf(e, sizeof e, "E%c%0*d", ex < 0 ? '-' : '+', edig, std::abs(ex));
  else
    std::snprintf(e, sizeof e, "%c%0*d", ex < 0 ? '-' : '+', edig + 1, std::abs(ex));
  std::snprintf(b, sizeof b, "%*s", w,
                ((neg ? "-" : "") + std::string("0.") + digits + e).c_str());
  return b;
}

// Fortran Dw.d: as Ew.d with the exponent letter D
std::string fortran_d(double v, int w, int dd) {
  std::string r = fortran_e(v, w, dd, 2);
  const size_t k = r.find('E');
  if (k != std::string::npos) r[k] = 'D';
  return r;
}

void vtk_head(FILE* f, const char* title, bool time, double t, int istep) {
  std::fprintf(f, "# vtk DataFile Version 3.0\n%-30s\nASCII\nDATASET UNSTRUCTURED_GRID\n",
               title);
  if (time)
    std::fprintf(f,
                 "FIELD FieldData 4\nTIME_S 1 1 double\n%16.6f\nTIME_H 1 1 double\n%16.6f\n"
                 "TIME_D 1 1 double\n%16.6f\nCYCLE 1 1 int\n%9d\n",
                 t, t / 3600.0, t / (24.0 * 3600.0), istep);
}

// coor_vtk / elm_vtk: quad = all nodes and hexa20 / tetra10 cells (VTK types
// 25 / 24 in the node orders of elm_vtk), else the vertex mesh
int vtk_mesh(FILE* f, const pm_deck_s* d, bool quad, int* npts) {
  const int nen = d->nen, nenv = d->nenv;
  const bool vert = !quad && d->mk_quad;
  const int np = vert ? d->nnodev : d->nnode;
  *npts = np;
  std::fprintf(f, "POINTS %10d double\n", np);
  for (int i = 0; i < np; ++i) {
    for (int k = 0; k < 3; ++k) std::fputs(fortran_e(d->x[(size_t)3 * i + k], 15, 5, 2).c_str(), f);
    std::fputc('\n', f);
  }
  static const int hexa20_vtk[20] = {5, 6, 7, 8, 1, 2, 3, 4, 13, 14,
                                     15, 16, 9, 10, 11, 12, 17, 18, 19, 20};
  static const int tetra10_vtk[10] = {1, 2, 3, 4, 5, 8, 6, 7, 10, 9};
  const int nno = quad ? nen : nenv;
  std::fprintf(f, "CELLS %10d%10d\n", d->numel, d->numel * (nno + 1));
  for (int el = 0; el < d->numel; ++el) {
    const int32_t* nd = &d->ix[(size_t)(nen + 1) * el];
    std::fprintf(f, "%10d", nno);
    for (int k = 0; k < nno; ++k) {
      const int slot = !quad ? k : nen == 20 ? hexa20_vtk[k] - 1 : tetra10_vtk[k] - 1;
      std::fprintf(f, "%10d", nd[slot] - 1);
    }
    std::fputc('\n', f);
  }
  const int type = quad ? (nen == 20 ? 25 : 24) : (nen == 20 ? 12 : 10);
  std::fprintf(f, "CELL_TYPES %10d\n", d->numel);
  for (int el = 0; el < d->numel; ++el) std::fprintf(f, "%3d\n", type);
  return PM_OK;
}

void vtk_point_int(FILE* f, const char* name, const int32_t* a, int np, int gdl) {
  std::fprintf(f, "SCALARS %-15s %-8s %3d\nLOOKUP_TABLE default\n", name, "int", gdl);
  for (int i = 0; i < np; ++i) {
    for (int j = 0; j < gdl; ++j) std::fprintf(f, "%10d", a[(size_t)gdl * i + j]);
    std::fputc('\n', f);
  }
}

void vtk_point_real(FILE* f, const char* name, const double* a, int np, int gdl, int stride) {
  std::fprintf(f, "SCALARS %-15s %-8s %3d\nLOOKUP_TABLE default\n", name, "double", gdl);
  for (int i = 0; i < np; ++i) {
    for (int j = 0; j < gdl; ++j)
      std::fputs(fortran_e(a[(size_t)stride * i + j], 15, 5, 3).c_str(), f);
    std::fputc('\n', f);
  }
}

void vtk_vectors(FILE* f, const char* name, const double* a, int np, int stride) {
  std::fprintf(f, "VECTORS %-15s double\n", name);
  for (int i = 0; i < np; ++i) {
    for (int j = 0; j < 3; ++j)
      std::fputs(fortran_e(a[(size_t)stride * i + j], 15, 5, 3).c_str(), f);
    std::fputc('\n', f);
  }
}

// make_full_tensor (Write_vtk.f:2310-2387): (xx, yy, zz, xy, yz, xz) -> 3 x 3
void vtk_tensors(FILE* f, const char* name, const double* t, int np) {
  std::fprintf(f, "TENSORS %-15s double\n", name);
  static const int map[9] = {0, 3, 5, 3, 1, 4, 5, 4, 2};
  for (int i = 0; i < np; ++i) {
    for (int j = 0; j < 9; ++j)
      std::fputs(fortran_e(t[(size_t)kNtn * i + map[j]], 15, 5, 3).c_str(), f);
    std::fputc('\n', f);
  }
}

void vtk_cell_int(FILE* f, const char* name, const int32_t* a, int n, int gdl) {
  std::fprintf(f, " SCALARS %-15s int %11d\nLOOKUP_TABLE default\n", name, gdl);
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < gdl; ++j) std::fprintf(f, "%10d", a[(size_t)gdl * i + j]);
    std::fputc('\n', f);
  }
}

void vtk_cells_common(FILE* f, const pm_deck_s* d) {
  std::fprintf(f, "CELL_DATA %9d\n", d->numel);
  std::vector<int32_t> v(d->numel);
  for (int el = 0; el < d->numel; ++el) v[el] = d->ix[(size_t)(d->nen + 1) * el + d->nen];
  vtk_cell_int(f, "mat", v.data(), d->numel, 1);
  for (int el = 0; el < d->numel; ++el) v[el] = el + 1;
  vtk_cell_int(f, "elIdG", v.data(), d->numel, 1);
}

// mid-side values as the average of their edge's vertices (split_u_p,
// mk_field_quad)
void quad_fill(const pm_deck_s* d, std::vector<double>& a, int gdl) {
  if (!d->mk_quad) return;
  for_edges(d, [&](int p, int q, int m) {
    for (int k = 0; k < gdl; ++k)
      a[(size_t)gdl * m + k] = 0.5 * (a[(size_t)gdl * p + k] + a[(size_t)gdl * q + k]);
  });
}

// write_mesh_geo_pm (Write_vtk.f:210-700): the mesh as read, <prefix>_bc.vtk
int write_geo(const pm_deck_s* d, const std::string& prefix, bool quad) {
  const std::string fn = prefix + "_bc.vtk";
  FILE* f = std::fopen(fn.c_str(), "w");
  if (!f) {
    g_err = "cannot write " + fn;
    return PM_E_ARG;
  }
  vtk_head(f, "Geometria lida", false, 0.0, 0);
  int np = 0;
  vtk_mesh(f, d, quad, &np);
  std::fprintf(f, "POINT_DATA %9d\n", np);
  std::vector<int32_t> ids(np);
  for (int i = 0; i < np; ++i) ids[i] = i + 1;
  vtk_point_int(f, "noIdG", ids.data(), np, 1);
  for (const std::string& m : d->node_macros) {
    if (m == "constrainpmec" || m == "constraindisp") {
      vtk_point_int(f, m.c_str(), d->id.data(), np, kNdf);
    } else if (m == "nodalforces") {
      vtk_point_real(f, "forces", d->f.data(), np, kNdf, kNdf);
    } else if (m == "nodalloads") {
      vtk_point_int(f, "nodalloads", d->nload.data(), np, kNdf);
    } else if (m == "initialpres") {
      std::vector<double> p(d->nnode);
      for (int i = 0; i < d->nnode; ++i) p[i] = d->u0[(size_t)kNdf * i + 3];
      if (quad) quad_fill(d, p, 1);
      vtk_point_real(f, "initialpres", p.data(), np, 1, 1);
    } else if (m == "initialstress") {
      vtk_tensors(f, "initialstress", d->tx0.data(), np);
    }
  }
  vtk_cells_common(f, d);
  for (const std::string& m : d->cell_macros)
    vtk_cell_int(f, m.c_str(), m == "elmtloads" ? d->eload.data() : d->eloadp.data(), d->numel, 7);
  std::fclose(f);
  return PM_OK;
}

// write_mesh_res_pm (Write_vtk.f:912-1399): <prefix>_istep_<n>.vtk
int write_res(const pm_deck_s* d, pm_handle h, const std::string& prefix, int istep, double t,
              bool quad, int fields) {
  const int nn = d->nnode;
  std::vector<double> u((size_t)kNdf * nn), dp(nn), poro(nn);
  std::vector<double> tx((size_t)kNtn * nn), txb((size_t)kNtn * nn), txe((size_t)kNtn * nn),
      fl((size_t)3 * nn);
  int st;
  if ((st = pm_get_state(h, u.data(), nullptr, dp.data())) != PM_OK) return st;
  if ((fields & 0x1e) && (st = pm_stress(h, tx.data(), txb.data(), txe.data(), fl.data())) != PM_OK)
    return st;
  if ((fields & 0x20) && (st = pm_get_porosity(h, poro.data())) != PM_OK) return st;
  if (d->fstress0 && (fields & 0x0e)) {
    for (size_t q = 0; q < tx.size(); ++q) {
      tx[q] += d->tx0[q];
      txb[q] += d->tx0[q];
    }
    for (int i = 0; i < nn; ++i)
      for (int k = 0; k < kNtn; ++k)
        txe[(size_t)kNtn * i + k] = tx[(size_t)kNtn * i + k] + (k < 3 ? u[(size_t)kNdf * i + 3] : 0.0);
  }
  const std::string fn = prefix + "_istep_" + std::to_string(istep) + ".vtk";
  FILE* f = std::fopen(fn.c_str(), "w");
  if (!f) {
    g_err = "cannot write " + fn;
    return PM_E_ARG;
  }
  vtk_head(f, "Malha poro mec", true, t, istep);
  int np = 0;
  vtk_mesh(f, d, quad, &np);
  vtk_cells_common(f, d);
  std::fprintf(f, "POINT_DATA %9d\n", np);
  std::vector<int32_t> ids(np);
  for (int i = 0; i < np; ++i) ids[i] = i + 1;
  vtk_point_int(f, "noIdG", ids.data(), np, 1);
  vtk_vectors(f, "desloc", u.data(), np, kNdf);
  std::vector<double> p(nn);
  for (int i = 0; i < nn; ++i) p[i] = u[(size_t)kNdf * i + 3];
  if (quad) quad_fill(d, p, 1);
  vtk_point_real(f, "pressao", p.data(), np, 1, 1);
  if (fields & 0x01) {
    if (quad) quad_fill(d, dp, 1);
    vtk_point_real(f, "deltaPressao", dp.data(), np, 1, 1);
  }
  if (fields & 0x20) {
    if (quad) quad_fill(d, poro, 1);
    vtk_point_real(f, "porosity", poro.data(), np, 1, 1);
  }
  if (fields & 0x10) {
    if (quad) quad_fill(d, fl, 3);
    vtk_vectors(f, "darcyFlux", fl.data(), np, 3);
  }
  if (quad && (fields & 0x0e)) {
    quad_fill(d, tx, kNtn);
    quad_fill(d, txe, kNtn);
    quad_fill(d, txb, kNtn);
  }
  if (fields & 0x02) vtk_tensors(f, "totalStress", tx.data(), np);
  if (fields & 0x04) vtk_tensors(f, "terzaghiStress", txe.data(), np);
  if (fields & 0x08) vtk_tensors(f, "BiotStress", txb.data(), np);
  std::fclose(f);
  return PM_OK;
}

}  // namespace

extern "C" {

int pm_deck_read(const char* path, pm_deck* out) {
  if (!path || !out) return PM_E_ARG;
  *out = nullptr;
  std::unique_ptr<pm_deck_s> d(new (std::nothrow) pm_deck_s());
  if (!d) return PM_E_NOMEM;
  d->path = path;
  d->dir = dir_of(path);
  Reader r;
  if (!r.push(path)) {
    g_err = r.err;
    return PM_E_ARG;
  }
  g_err.clear();
  if (!parse(r, d.get())) return PM_E_ARG;
  *out = d.release();
  return PM_OK;
}

const char* pm_deck_error(void) { return g_err.c_str(); }

void pm_deck_free(pm_deck d) { delete d; }

int pm_deck_value(pm_deck d, const char* name, double* v) {
  if (!d || !name || !v) return PM_E_ARG;
  const std::string n = name;
  const Settings& s = d->run0;
  const std::map<std::string, double> vals = {
      {"nnode", d->nnode}, {"nnodev", d->nnodev}, {"numel", d->numel}, {"numat", d->numat},
      {"nen", d->nen}, {"nenv", d->nenv}, {"nloads", d->nloads}, {"maxt", d->maxt},
      {"fstress0", d->fstress0}, {"mk_quad", d->mk_quad}, {"reord", d->reord},
      {"solver", s.solver},
      {"precond", s.precond}, {"maxit", s.maxit}, {"solvtol", s.solvtol},
      {"maxnlit", s.maxnlit}, {"tol", s.tol}, {"stop_crit", s.stop_crit},
      {"nkrylov", s.nkrylov}, {"dt", s.dt}, {"gravity_x", s.gravity[0]},
      {"gravity_y", s.gravity[1]}, {"gravity_z", s.gravity[2]},
      {"nprint", (double)d->print_nodes.size()}, {"nops", (double)d->prog.size()},
      {"unknown_macros", d->nunknown}};
  auto it = vals.find(n);
  if (it == vals.end()) return PM_E_ARG;
  *v = it->second;
  return PM_OK;
}

int pm_deck_int_array(pm_deck d, const char* name, const int32_t** p, int64_t* n) {
  if (!d || !name || !p || !n) return PM_E_ARG;
  const std::map<std::string, const std::vector<int32_t>*> a = {
      {"ix", &d->ix}, {"ie", &d->ie}, {"id", &d->id}, {"nload", &d->nload},
      {"eload", &d->eload}, {"eloadp", &d->eloadp}, {"fnno", &d->fnno}, {"load", &d->load},
      {"print_nodes", &d->print_nodes}};
  auto it = a.find(name);
  if (it == a.end()) return PM_E_ARG;
  *p = it->second->data();
  *n = (int64_t)it->second->size();
  return PM_OK;
}

int pm_deck_real_array(pm_deck d, const char* name, const double** p, int64_t* n) {
  if (!d || !name || !p || !n) return PM_E_ARG;
  const std::map<std::string, const std::vector<double>*> a = {
      {"e", &d->e}, {"x", &d->x}, {"f", &d->f}, {"u0", &d->u0}, {"tx0", &d->tx0},
      {"fload", &d->fload}};
  auto it = a.find(name);
  if (it == a.end()) return PM_E_ARG;
  *p = it->second->data();
  *n = (int64_t)it->second->size();
  return PM_OK;
}

int pm_deck_create(pm_deck d, pm_handle* h) {
  if (!d || !h) return PM_E_ARG;
  // the mesh macro numbers the equations in reord's node order (Main.f:585-590)
  std::vector<int32_t> num;
  if (d->reord) {
    num.resize(d->nnode);
    int st = pm_reord(d->nnode, d->numel, d->nen, d->ix.data(), num.data());
    if (st != PM_OK) return st;
  }
  int st = pm_mesh_create(d->nnode, d->nnodev, d->numel, d->nen, d->nenv, 3, kNdf, d->ix.data(),
                          d->id.data(), d->fnno.data(), d->x.data(), d->numat, d->ie.data(),
                          d->e.data(), d->reord ? num.data() : nullptr, h);
  if (st != PM_OK) return st;
  std::vector<double> zero(d->nnode, 0.0);
  if ((st = pm_set_loads(*h, d->eload.data(), d->eloadp.data(), d->nload.data(), d->f.data(),
                         d->nloads, d->maxt, d->nloads ? d->load.data() : nullptr,
                         d->nloads ? d->fload.data() : nullptr)) != PM_OK ||
      (st = pm_set_env(*h, d->init.gravity, d->init.dt, 0.0, 0)) != PM_OK ||
      (st = pm_set_state(*h, d->u0.data(), d->u0.data(), zero.data())) != PM_OK ||
      (st = pm_set_nkrylov(*h, d->init.nkrylov)) != PM_OK ||
      (d->fstress0 && (st = pm_set_initial_stress(*h, d->tx0.data())) != PM_OK)) {
    pm_destroy(*h);
    *h = nullptr;
  }
  return st;
}

int pm_deck_run(pm_deck d, pm_handle h, const char* prefix, int format, int* nsteps) {
  if (!d || !h || !prefix || (format != 0 && format != 1)) return PM_E_ARG;
  g_err.clear();
  Printer pr{prefix, format, {}};
  Settings s = d->init;
  int istep = 0;
  double t = 0.0;
  const int nn = d->nnode;
  std::vector<double> u((size_t)kNdf * nn), u0((size_t)kNdf * nn), dp(nn), poro(nn);
  std::vector<double> tx((size_t)kNtn * nn), txb((size_t)kNtn * nn), txe((size_t)kNtn * nn),
      fl((size_t)3 * nn);
  struct Frame {
    size_t start;
    int left;
  };
  std::vector<Frame> loops;
  bool log_open = false;
  int st = PM_OK;
  double phase_s[4] = {0, 0, 0, 0}, tform_s = 0.0;  // ELMT parts, SOLVR; TFORM
  const auto wall0 = std::chrono::steady_clock::now();
  for (size_t pc = 0; pc < d->prog.size(); ++pc) {
    const Op& op = d->prog[pc];
    switch (op.kind) {
      case OP_DT:
      case OP_NL:
      case OP_SOLVER:
      case OP_GRAVITY:
        s = op.s;
        if ((st = pm_set_env(h, s.gravity, s.dt, t, istep)) != PM_OK ||
            (st = pm_set_nkrylov(h, s.nkrylov)) != PM_OK)
          return st;
        break;
      case OP_LOOP:
        if (op.n <= 0) {
          int depth = 1;  // skip to the matching 'next'
          while (depth && ++pc < d->prog.size())
            depth += d->prog[pc].kind == OP_LOOP ? 1 : d->prog[pc].kind == OP_NEXT ? -1 : 0;
        } else {
          loops.push_back({pc, op.n});
        }
        break;
      case OP_NEXT:
        if (--loops.back().left > 0) pc = loops.back().start;
        else loops.pop_back();
        break;
      case OP_SOLV: {
        pm_step_info info;
        if ((st = pm_step(h, s.maxnlit, s.tol, s.stop_crit, s.solver, s.precond, s.solvtol,
                          s.maxit, 1, &info)) != PM_OK)
          return st;
        istep += 1;
        t = t + s.dt;
        // the solver log (Iters.f 'flog' lines; the layout of the shipped
        // golden logs): iterations, energy norm x.Kx, tolerance, seconds
        double tm[8] = {0};
        pm_get_timers(h, tm, 8);
        for (int q = 0; q < 4; ++q) phase_s[q] += tm[q] * 1e-3;
        const std::string ln = std::string(prefix) + "_log_1.txt";
        FILE* lf = std::fopen(ln.c_str(), log_open ? "a" : "w");
        if (!lf) {
          g_err = "cannot write " + ln;
          return PM_E_ARG;
        }
        if (!log_open) std::fputs("Solver control flop.\n", lf);
        log_open = true;
        static const char* names[] = {"", "PCG:", "GMRES2:", "", "", "", "", "MINRES:", "", "",
                                      "", "RPSQMR:"};
        const char* nm = s.solver >= 0 && s.solver < 12 && names[s.solver][0] ? names[s.solver]
                                                                               : "SOLVER:";
        std::fprintf(lf, "%s  it %9d energy norm %s tol %s time %20.2f\n", nm, info.iters,
                     fortran_d(info.xkx, 20, 10).c_str(), fortran_d(s.solvtol, 20, 10).c_str(),
                     tm[3] * 1e-3);
        std::fclose(lf);
        break;
      }
      case OP_PNUP:
        if ((st = pm_get_state(h, u.data(), nullptr, nullptr)) != PM_OK) return st;
        for (int n : d->print_nodes)
          if (n >= 1 && n <= nn &&
              (st = pr.print("up", "DeslocAndPress", n, istep, t, &u[(size_t)kNdf * (n - 1)],
                             kNdf)) != PM_OK)
            return st;
        break;
      case OP_PNSF: {
        const auto ts0 = std::chrono::steady_clock::now();
        if ((st = pm_stress(h, tx.data(), txb.data(), txe.data(), fl.data())) != PM_OK ||
            (st = pm_get_state(h, u.data(), nullptr, nullptr)) != PM_OK ||
            (st = pm_get_porosity(h, poro.data())) != PM_OK)
          return st;
        tform_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - ts0).count();
        if (d->fstress0) {
          // pnsf adds the initial stress (Main.f:2360-2370), then effective_stress
          for (size_t q = 0; q < tx.size(); ++q) {
            tx[q] += d->tx0[q];
            txb[q] += d->tx0[q];
          }
          for (int i = 0; i < nn; ++i)
            for (int k = 0; k < kNtn; ++k)
              txe[(size_t)kNtn * i + k] =
                  tx[(size_t)kNtn * i + k] + (k < 3 ? u[(size_t)kNdf * i + 3] : 0.0);
        }
        const bool gold = format == 1;
        for (int n : d->print_nodes) {
          if (n < 1 || n > nn) continue;
          const size_t i = n - 1;
          if ((st = pr.print("stress", gold ? "stressTotal" : "totalStress", n, istep, t,
                             &tx[kNtn * i], kNtn)) != PM_OK ||
              (st = pr.print("stressE", gold ? "stressE" : "eSstress", n, istep, t,
                             &txe[kNtn * i], kNtn)) != PM_OK ||
              (st = pr.print("stressB", gold ? "stressBiot" : "biotStress", n, istep, t,
                             &txb[kNtn * i], kNtn)) != PM_OK ||
              (st = pr.print("flux", gold ? "stressFlux" : "darcyFlux", n, istep, t, &fl[3 * i],
                             3)) != PM_OK ||
              (st = pr.print("poro", "poro", n, istep, t, &poro[i], 1)) != PM_OK)
            return st;
        }
        break;
      }
      case OP_PGEO:
        if ((st = write_geo(d, prefix, false)) != PM_OK) return st;
        break;
      case OP_PRES:
        if ((st = write_res(d, h, prefix, istep, t, true, 0x3f)) != PM_OK) return st;
        break;
      case OP_STOP:
        pc = d->prog.size();
        break;
    }
  }
  if (nsteps) *nsteps = istep;
  // the run's log (write_log_file, Write_log.f:46-408): phase times in
  // seconds, then the sizes of the mesh and of the linear system
  int neq = 0, nc = 0;
  int64_t nad = 0, nnz = 0;
  if ((st = pm_get_sizes(h, &neq, &nad, &nc, &nnz)) != PM_OK) return st;
  const double wall =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
  const std::string tn = std::string(prefix) + "_t_1.txt";
  FILE* tf = std::fopen(tn.c_str(), "w");
  if (!tf) {
    g_err = "cannot write " + tn;
    return PM_E_ARG;
  }
  std::fprintf(tf, "# Arquivo de log do poro mecanico\nTempos (seg):\n"
                   "Resolucao do tempo:  1.00E-06\n");
  const std::pair<const char*, double> rows[] = {
      {"ELMT", phase_s[0] + phase_s[1] + phase_s[2]}, {"TFORM", tform_s},
      {"SOLVR", phase_s[3]}, {"COLOR", 0.0}, {"TOTAL", wall}};
  for (const auto& r : rows) std::fprintf(tf, "%-6s%18.6f\n", r.first, r.second);
  std::fprintf(tf, "Malha e sistema linear:\nPoromecanico:\n");
  const std::pair<const char*, long long> cnt[] = {
      {"neq", neq}, {"nad", (long long)nad}, {"nnode", d->nnode}, {"numel", d->numel},
      {"colors", nc}};
  for (const auto& r : cnt) std::fprintf(tf, "%-6s%16lld\n", r.first, r.second);
  std::fclose(tf);
  return PM_OK;
}

int pm_deck_write_geo(pm_deck d, const char* prefix, int quad) {
  if (!d || !prefix) return PM_E_ARG;
  return write_geo(d, prefix, quad != 0);
}

int pm_deck_write_res(pm_deck d, pm_handle h, const char* prefix, int istep, double t, int quad,
                      int fields) {
  if (!d || !h || !prefix) return PM_E_ARG;
  return write_res(d, h, prefix, istep, t, quad != 0, fields);
}

}  // extern "C"
