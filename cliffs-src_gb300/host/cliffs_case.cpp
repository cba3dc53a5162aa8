// cliffs_case.cpp -- the reference driver's setup (see cliffs_case.hpp).
#include "cliffs_case.hpp"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <sstream>

#include "nc3.hpp"

namespace cliffs_host {
namespace {

// Fortran list-directed read of the next record: the leading values of the
// line, the rest ignored.
class ParamReader {
 public:
  explicit ParamReader(const std::string& path) : in_(path) {
    if (!in_) throw CaseError("cannot open parameter file " + path);
  }
  std::string line() {
    std::string s;
    if (!std::getline(in_, s)) throw CaseError("parameter file ends early");
    return s;
  }
  std::istringstream record() { return std::istringstream(line()); }
  double real() {
    auto r = record();
    std::string tok;
    r >> tok;
    return to_double(tok);
  }
  int integer() { return (int)std::lround(real()); }
  // format (a): the whole line; a file name has no blanks
  std::string name() {
    auto r = record();
    std::string tok;
    r >> tok;
    if (tok.empty()) throw CaseError("missing file name in parameter file");
    return tok;
  }
  static double to_double(std::string tok) {
    for (char& c : tok)
      if (c == 'd' || c == 'D') c = 'e';  // Fortran exponent letter
    try {
      size_t used = 0;
      const double v = std::stod(tok, &used);
      return v;
    } catch (...) {
      throw CaseError("bad number in parameter file: '" + tok + "'");
    }
  }

 private:
  std::ifstream in_;
};

std::vector<double> read_vector(const nc3::Reader& f, int varid, const std::string& what) {
  const nc3::Var& v = f.var(varid);
  if (v.type != nc3::FLOAT && v.type != nc3::DOUBLE) throw CaseError(what + " unexpected type");
  return f.get_double(varid);
}

// MasterGrid.f and NestedGrid.f read variables 1, 2, 3 as x, y and depth.
// Writers other than the NetCDF library may store them in another order, so
// they are found by shape: x on dimension 1, y on dimension 2, depth on (y, x);
// files in the reference's order give the same ids.
void grid_vars(const nc3::Reader& f, int* xid, int* yid, int* zid) {
  *xid = *yid = *zid = -1;
  for (int i = 0; i < f.nvars(); ++i) {
    const std::vector<int32_t>& d = f.var(i).dims;
    if (d.size() == 1 && d[0] == 0 && *xid < 0) *xid = i;
    else if (d.size() == 1 && d[0] == 1 && *yid < 0) *yid = i;
    else if (d.size() == 2 && d[0] == 1 && d[1] == 0 && *zid < 0) *zid = i;
  }
  if (*xid < 0 || *yid < 0) {
    *xid = 0;
    *yid = 1;
  }
  if (*zid < 0) *zid = 2;
}

bool exists(const std::string& path) {
  std::ifstream f(path);
  return (bool)f;
}

double absmax_eta(const std::vector<double>& recs, int len, int rec) {
  // (nt, 3, len): component 3 (eta) of record rec
  double w = 0;
  const double* p = recs.data() + ((size_t)rec * 3 + 2) * (size_t)len;
  for (int k = 0; k < len; ++k) w = std::max(w, std::fabs(p[k]));
  return w;
}

}  // namespace

void pinpoint(const double* xx, int n, double xp, int32_t* ip_out, double* cp) {
  int ip = 1, ipp = n;
  while (ip + 2 <= ipp) {
    const int med = (ip + ipp) / 2;
    if (xp > xx[med - 1])
      ip = med;
    else
      ipp = med;
  }
  *ip_out = ip;
  *cp = n > 1 ? (xx[ip] - xp) / (xx[ip] - xx[ip - 1]) : 0.5;
}

void apply_initial_conditions(int nxq, int nyq, const double* xq, const double* yq, const double* q,
                              int nxp, int nyp, const double* xp, const double* yp, double* p) {
  const double zero = 0.1e-20;
  const double x1 = xq[0] - zero, x2 = xq[nxq - 1] + zero;
  const double y1 = yq[0] - zero, y2 = yq[nyq - 1] + zero;
  auto Q = [&](int i, int j) { return q[(size_t)(j - 1) * nxq + (i - 1)]; };  // 1-based
  if (nxq > 2 && nyq > 2) {
    for (int i = 0; i < nxp; ++i) {
      const double xx = xp[i];
      if (!(xx >= x1 && xx <= x2)) continue;
      int32_t ii;
      double xcc;
      pinpoint(xq, nxq, xx, &ii, &xcc);
      for (int j = 0; j < nyp; ++j) {
        const double yy = yp[j];
        if (!(yy >= y1 && yy <= y2)) continue;
        int32_t jj;
        double ycc;
        pinpoint(yq, nyq, yy, &jj, &ycc);
        const double v = (Q(ii, jj) * xcc + Q(ii + 1, jj) * (1 - xcc)) * ycc +
                         (Q(ii, jj + 1) * xcc + Q(ii + 1, jj + 1) * (1 - xcc)) * (1 - ycc);
        p[(size_t)j * nxp + i] += v;
      }
    }
  }
  if (nyq == 1 && nxq > 2) {
    for (int i = 0; i < nxp; ++i) {
      const double xx = xp[i];
      if (!(xx >= x1 && xx <= x2)) continue;
      int32_t ii;
      double xcc;
      pinpoint(xq, nxq, xx, &ii, &xcc);
      const double v = Q(ii, 1) * xcc + Q(ii + 1, 1) * (1 - xcc);
      for (int j = 0; j < nyp; ++j) p[(size_t)j * nxp + i] += v;
    }
  }
  if (nxq == 1 && nyq > 2) {
    for (int j = 0; j < nyp; ++j) {
      const double yy = yp[j];
      if (!(yy >= y1 && yy <= y2)) continue;
      int32_t jj;
      double ycc;
      pinpoint(yq, nyq, yy, &jj, &ycc);
      const double v = Q(1, jj) * ycc + Q(1, jj + 1) * (1 - ycc);
      for (int i = 0; i < nxp; ++i) p[(size_t)j * nxp + i] += v;
    }
  }
}

Case read_case(const std::string& srcdir, const std::string& bprfx, const std::string& aprfx,
               const std::string& paramdir, const std::string& paramfile) {
  Case c;
  Params& p = c.p;
  ParamReader pr(paramdir + paramfile);
  // ---- allabout.f / MasterGrid.f
  p.cartesian = pr.integer() == 1;
  c.log.push_back(p.cartesian ? "CARTESIAN COORDINATE SYSTEM" : "SPHERICAL (LON,LAT) COORDINATE SYSTEM");
  p.master_path = pr.name();
  {
    const size_t slash = p.master_path.rfind('/');
    const size_t a = slash == std::string::npos ? 0 : slash + 1;
    const size_t b = p.master_path.find(".nc");
    p.master_name = p.master_path.substr(a, (b == std::string::npos ? p.master_path.size() : b) - a);
    const std::string fname = paramdir + p.master_path;
    c.log.push_back("Master bathy/topo file:  " + fname);
    nc3::Reader f(fname);
    if (f.ndims() < 2 || f.nvars() < 3) throw CaseError("master grid file needs 2 dimensions and 3 variables");
    c.nx = (int)f.dim_len(0);
    c.ny = (int)f.dim_len(1);
    int xid, yid, zid;
    grid_vars(f, &xid, &yid, &zid);
    c.x = read_vector(f, xid, "x-vector");
    c.y = read_vector(f, yid, "y-vector");
    c.dep = read_vector(f, zid, "bathy/topo");
    if ((int)c.x.size() != c.nx || (int)c.y.size() != c.ny || (int64_t)c.dep.size() != (int64_t)c.nx * c.ny)
      throw CaseError("master grid variables do not match its dimensions");
    if (f.nvars() > 3) {  // MasterGrid.f:118-120: a fourth variable, the last
      int last = f.nvars() - 1;
      if (last == xid || last == yid || last == zid)
        for (int i = 0; i < f.nvars(); ++i)
          if (i != xid && i != yid && i != zid) last = i;
      c.zeta = f.get_double(last);
      c.has_zeta = true;
      if ((int)c.zeta.size() < c.ny) throw CaseError("width term shorter than the y axis");
      c.zeta.resize(c.ny);
    }
    c.log.push_back("grid size " + std::to_string(c.nx) + " " + std::to_string(c.ny));
  }
  p.nests = pr.integer();
  if (p.nests > 0 && (c.nx < 3 || c.ny < 3)) throw CaseError("nesting in 1D is not permitted");
  if (p.nests < 0 || p.nests > 99) throw CaseError("number of nested grids out of range");
  // ---- NestedGrid.f
  for (int ns = 0; ns < p.nests; ++ns) {
    Nest n;
    const std::string path = pr.name();
    const size_t b = path.find(".nc");
    n.name = path.substr(0, b == std::string::npos ? path.size() : b);
    p.child_paths.push_back(path);
    p.child_names.push_back(n.name);
    nc3::Reader f(paramdir + path);
    n.mm = (int32_t)f.dim_len(0);
    n.nn = (int32_t)f.dim_len(1);
    int xid, yid, zid;
    grid_vars(f, &xid, &yid, &zid);
    n.x = read_vector(f, xid, "child x-vector");
    n.y = read_vector(f, yid, "child y-vector");
    if ((int)n.x.size() != n.mm || (int)n.y.size() != n.nn) throw CaseError("child grid axes do not match");
    if (n.x.front() < c.x.front() || n.x.back() > c.x.back() || n.y.front() < c.y.front() ||
        n.y.back() > c.y.back())
      throw CaseError("grid " + std::to_string(ns + 1) + " not within Master grid limits");
    pinpoint(c.y.data(), c.ny, n.y.front(), &n.S_ny, &n.S_cy);
    pinpoint(c.y.data(), c.ny, n.y.back(), &n.N_ny, &n.N_cy);
    n.SN_nx.resize(n.mm);
    n.SN_cx.resize(n.mm);
    for (int i = 0; i < n.mm; ++i) pinpoint(c.x.data(), c.nx, n.x[i], &n.SN_nx[i], &n.SN_cx[i]);
    pinpoint(c.x.data(), c.nx, n.x.front(), &n.W_nx, &n.W_cx);
    pinpoint(c.x.data(), c.nx, n.x.back(), &n.E_nx, &n.E_cx);
    n.WE_ny.resize(n.nn);
    n.WE_cy.resize(n.nn);
    for (int i = 0; i < n.nn; ++i) pinpoint(c.y.data(), c.ny, n.y[i], &n.WE_ny[i], &n.WE_cy[i]);
    c.log.push_back("nested Grid " + std::to_string(ns + 1) + " " + path + " " + std::to_string(n.mm) + " " +
                    std::to_string(n.nn));
    c.nests.push_back(std::move(n));
  }
  p.cuke = pr.real();
  p.ground = pr.real();
  p.crough = pr.real();
  p.itopo = pr.integer();
  p.dwall = pr.real();
  p.dt = pr.real();
  p.steps_total = pr.integer();
  p.quake = pr.integer();
  p.freeze = pr.integer() == 0;
  p.seaout = pr.integer();
  p.lonsub = pr.integer();
  p.latsub = pr.integer();
  p.bndout = pr.integer();
  p.maxout = pr.integer();
  p.ngages = pr.integer();
  if (p.ngages >= 1) {
    p.gout = pr.integer();
    for (int k = 0; k < p.ngages; ++k) {
      auto r = pr.record();
      std::string a, b;
      r >> a >> b;
      if (b.empty()) throw CaseError("gage line needs I and J");
      p.gage_i.push_back((int32_t)std::lround(ParamReader::to_double(a)));
      p.gage_j.push_back((int32_t)std::lround(ParamReader::to_double(b)));
    }
  }
  if (!(p.dt > 0)) throw CaseError("time step must be positive");
  if (p.seaout < 1 || p.bndout < 1 || p.maxout < 1 || (p.ngages >= 1 && p.gout < 1))
    throw CaseError("output intervals must be positive");
  if (p.lonsub < 1 || p.latsub < 1) throw CaseError("subsampling must be positive");
  for (int k = 0; k < p.ngages; ++k)
    if (p.gage_i[k] < 1 || p.gage_i[k] > c.nx || p.gage_j[k] < 1 || p.gage_j[k] > c.ny)
      throw CaseError("gage " + std::to_string(k + 1) + " outside the grid");
  // ---- cliffs_main.f:131-137: vertical wall at dwall
  if (p.itopo == 0)
    for (double& d : c.dep)
      if (d <= p.dwall) d = -999;
  // ---- 1-D and 2-D (cliffs_main.f:140-164)
  c.xrun = c.nx > 2;
  c.yrun = c.ny > 2;
  if (!c.xrun) p.lonsub = 1;
  if (!c.yrun) p.latsub = 1;
  if (!c.xrun && !c.yrun) throw CaseError("grid needs more than 2 nodes along x or y");
  if (bprfx == "0" && aprfx == "0") throw CaseError("no input of any kind");
  // ---- get_boundary_feed.f
  if (bprfx != "0") {
    const std::string base = srcdir + bprfx + "_" + p.master_name;
    c.log.push_back(" Boundary Input:");
    auto load = [&](const std::string& side, int len, std::vector<double>& recs, bool take_time) {
      const std::string fname = base + "_" + side + ".nc";
      c.log.push_back(fname);
      if (!exists(fname)) throw CaseError("not found: " + fname);
      nc3::Reader f(fname);
      // get_boundary_feed.f takes the lengths of dimensions 1 and 3 (pnt,
      // tim as opennc4feed.f defines them); here they are taken from the
      // records variable vals(tim, uvq, pnt) itself, whatever the order in
      // which the writer defined its dimensions
      if (f.nvars() < 2 || f.var(0).dims.size() != 3) throw CaseError("unexpected layout of " + fname);
      const int n = (int)f.dim_len(f.var(0).dims[2]), nt = (int)f.dim_len(f.var(0).dims[0]);
      if (n != len) throw CaseError("size mismatch: expected " + std::to_string(len) + " provided " + std::to_string(n));
      if (take_time) {
        c.nt = nt;
        if (nt < 2) throw CaseError("unsufficient time-series length: " + std::to_string(nt) + " samples");
        c.tinput = f.get_double(1);
      } else if (nt != c.nt) {
        throw CaseError("size mismatch in " + fname);
      }
      recs = f.get_double(0);
      if ((int64_t)recs.size() != (int64_t)c.nt * 3 * len) throw CaseError("record size mismatch in " + fname);
    };
    if (c.xrun) {
      load("west", c.ny, c.west, true);
      load("east", c.ny, c.east, false);
    }
    if (c.yrun) {
      load("south", c.nx, c.south, !c.xrun);
      load("north", c.nx, c.north, false);
    }
    // first record whose edge elevation reaches the still-sea threshold
    int it = 1;
    double wave = 0;
    for (it = 1; it <= c.nt; ++it) {
      double w = 0;
      if (c.xrun) w = std::max({w, absmax_eta(c.west, c.ny, it - 1), absmax_eta(c.east, c.ny, it - 1)});
      if (c.yrun) w = std::max({w, absmax_eta(c.south, c.nx, it - 1), absmax_eta(c.north, c.nx, it - 1)});
      wave = w;
      if (wave >= p.cuke) break;
    }
    if (it >= c.nt) throw CaseError("bndr signal below threshold");
    c.irec = it;
    c.feed_wave = wave;
    c.bndr_input = true;
  }
  // ---- get_initial_state.f
  c.H = c.dep;  // cel = dep (cliffs_main.f:190): the surface at rest
  c.u.assign(c.dep.size(), 0.0);
  c.v.assign(c.dep.size(), 0.0);
  if (aprfx != "0") {
    const std::string base = srcdir + aprfx;
    const std::string fh = base + "_h.nc", fu = base + "_u.nc", fv = base + "_v.nc";
    c.hinput = exists(fh);
    c.uinput = exists(fu);
    c.vinput = exists(fv);
    c.log.push_back("Initial displacement: " + fh + (c.hinput ? "" : " not found"));
    const std::string& first = c.hinput ? fh : c.uinput ? fu : fv;
    if (c.hinput || c.uinput || c.vinput) {
      nc3::Reader f(first);
      int ntsrc = 0, nxs = 0, nys = 0;
      for (int i = 0; i < f.ndims(); ++i) {
        const std::string n = f.dim(i).name.substr(0, 3);
        if (n == "tim") ntsrc = (int)f.dim_len(i);
        else if (n == "xxx" || n == "lon") nxs = (int)f.dim_len(i);
        else if (n == "yyy" || n == "lat") nys = (int)f.dim_len(i);
      }
      int tid = -1, xid = -1, yid = -1;
      for (int i = 0; i < f.nvars(); ++i) {
        const std::string n = f.var(i).name.substr(0, 3);
        if (n == "tim") tid = i;
        else if (n == "xxx" || n == "lon") xid = i;
        else if (n == "yyy" || n == "lat") yid = i;
      }
      if (tid < 0 || xid < 0 || yid < 0 || ntsrc < 1 || nxs < 1 || nys < 1)
        throw CaseError("initial state file lacks time, x or y: " + first);
      const std::vector<double> xs = f.get_double(xid), ys = f.get_double(yid), ts = f.get_double(tid);
      int isrc = 1;
      if (c.nt < 2) {
        c.tinput.assign(1, ts[0]);
        c.irec = 1;
      } else {
        int32_t ip;
        double cp;
        pinpoint(ts.data(), ntsrc, c.tinput[c.irec - 1], &ip, &cp);
        isrc = ip;
      }
      c.tsrc_used = ts[isrc - 1];
      auto field = [&](const std::string& path) {
        nc3::Reader g(path);
        const int vid = g.nvars() - 1;
        std::vector<double> a;
        if (g.var(vid).is_record) {
          a = g.get_records_double(vid, isrc - 1, 1);
        } else {  // a fixed (time, y, x) variable: take record isrc
          const std::vector<double> all = g.get_double(vid);
          const size_t per = (size_t)nxs * nys, off = (size_t)(isrc - 1) * per;
          if (all.size() < off + per) throw CaseError("initial state size mismatch in " + path);
          a.assign(all.begin() + off, all.begin() + off + per);
        }
        if ((int64_t)a.size() != (int64_t)nxs * nys) throw CaseError("initial state size mismatch in " + path);
        for (double& x : a)
          if (x < -1.0e+10) x = 0;  // no-data marker
        return a;
      };
      if (c.uinput)
        apply_initial_conditions(nxs, nys, xs.data(), ys.data(), field(fu).data(), c.nx, c.ny, c.x.data(),
                                 c.y.data(), c.u.data());
      if (c.vinput)
        apply_initial_conditions(nxs, nys, xs.data(), ys.data(), field(fv).data(), c.nx, c.ny, c.x.data(),
                                 c.y.data(), c.v.data());
      if (c.hinput) {
        std::vector<double> q = field(fh);
        if (p.quake == 1) {  // deform the bottom
          for (double& x : q) x = -x;
          apply_initial_conditions(nxs, nys, xs.data(), ys.data(), q.data(), c.nx, c.ny, c.x.data(), c.y.data(),
                                   c.dep.data());
        } else {  // deform the surface
          apply_initial_conditions(nxs, nys, xs.data(), ys.data(), q.data(), c.nx, c.ny, c.x.data(), c.y.data(),
                                   c.H.data());
        }
      }
    } else if (c.nt < 1) {
      throw CaseError("no initial state and no boundary input");
    }
  }
  if (c.nt < 2) p.freeze = false;
  if (c.tinput.empty()) throw CaseError("no start time");
  c.t0 = c.tinput[c.irec - 1];
  return c;
}

}  // namespace cliffs_host
