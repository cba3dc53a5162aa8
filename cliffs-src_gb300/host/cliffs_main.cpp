// cliffs_main.cpp -- the Cliffs driver (cliffs_main.f) on the GB300 library.
//
//   cliffs_gb300 <output dir/prefix> <source dir/> <boundary prefix, 0 for none>
//                <area prefix, 0 for none> <param dir/param file> [notes...]
//                [--dry-run]
//
// The same command line, parameter file, input files and output files as the
// reference's executable (cliffs_main.f:62-99, 232-290, 380-400):
//   <prefix>_log.txt, <prefix>_maxwave.nc, <prefix>_sea_{h,u,v}.nc,
//   <prefix>_gages.nc, <prefix>_<child>_{west,east,south,north}.nc.
// Setup is read on the host (cliffs_case.cpp); every time step, max-wave,
// gauge, screenshot and child-feed computation runs on the GPU through
// include/cliffs_gpu.h, with the fields resident on the device between output
// events.  --dry-run reads and checks the case, prints a JSON summary and
// writes the output files' headers with the initial records computed on the
// host, without a GPU.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <deque>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cliffs_gpu.h"
#include "cliffs_case.hpp"
#include "nc3.hpp"

using cliffs_host::Case;
using cliffs_host::CaseError;

namespace {

constexpr float kNan = -1.e32f;  // NAN of module MASTER (global_modules.f:18)

class Log {
 public:
  explicit Log(const std::string& path) : f_(path) {}
  template <typename T>
  Log& operator<<(const T& v) {
    f_ << v;
    return *this;
  }
  void line(const std::string& s) { f_ << ' ' << s << '\n' << std::flush; }
  bool ok() const { return (bool)f_; }

 private:
  std::ofstream f_;
};

std::string stamp() {
  std::time_t t = std::time(nullptr);
  char buf[64];
  std::strftime(buf, sizeof buf, "%Y/%m/%d %H:%M:%S", std::localtime(&t));
  return buf;
}

void check(int r, const char* what) {
  if (r < 0) throw std::runtime_error(std::string(what) + ": " + cliffs_gpu_strerror(r));
}

// ---- output files (opennc4*.f) --------------------------------------------

struct SeaFile {  // opennc4sea.f: one of ha, ua, va
  std::unique_ptr<nc3::Writer> w;
  int tvar = -1, var = -1;
};

SeaFile open_sea(const std::string& fname, int who, const std::vector<double>& lon, const std::vector<double>& lat,
                 bool cartesian) {
  SeaFile s;
  s.w.reset(new nc3::Writer(fname));
  nc3::Writer& w = *s.w;
  const std::string xn = cartesian ? "xxx" : "lon", yn = cartesian ? "yyy" : "lat";
  const int dx = w.def_dim(xn, (int64_t)lon.size()), dy = w.def_dim(yn, (int64_t)lat.size());
  const int dt = w.def_dim("time", 0);
  const int xv = w.def_var(xn, nc3::DOUBLE, {dx}), yv = w.def_var(yn, nc3::DOUBLE, {dy});
  s.tvar = w.def_var("time", nc3::DOUBLE, {dt});
  static const char* names[] = {"ha", "ua", "va"};
  static const char* longn[] = {"Surface Displacement", "U (zonal) Velocity", "V (meridional) Velocity"};
  static const char* units[] = {"meters", "meters/second", "meters/second"};
  s.var = w.def_var(names[who - 1], nc3::FLOAT, {dt, dy, dx});
  w.put_att_text(s.var, "name", longn[who - 1]);
  w.put_att_text(s.var, "units", units[who - 1]);
  if (cartesian) {
    w.put_att_text(xv, "name", "subset_x");
    w.put_att_text(xv, "units", "meters");
    w.put_att_text(yv, "name", "subset_y");
    w.put_att_text(yv, "units", "meters");
  } else {
    w.put_att_text(xv, "name", "subset_longitude");
    w.put_att_text(xv, "units", "degrees_east");
    w.put_att_text(yv, "name", "subset_latitude");
    w.put_att_text(yv, "units", "degrees_north");
  }
  w.put_att_text(s.tvar, "name", "time");
  w.put_att_text(s.tvar, "units", "seconds");
  w.enddef();
  w.put_var(xv, lon.data(), (int64_t)lon.size());
  w.put_var(yv, lat.data(), (int64_t)lat.size());
  return s;
}

struct MaxFile {  // opennc4max.f
  std::unique_ptr<nc3::Writer> w;
  int e = -1, v = -1;
};

MaxFile open_max(const std::string& fname, const Case& c) {
  MaxFile m;
  m.w.reset(new nc3::Writer(fname));
  nc3::Writer& w = *m.w;
  const bool cart = c.p.cartesian;
  const std::string xn = cart ? "xxx" : "lon", yn = cart ? "yyy" : "lat";
  const int dx = w.def_dim(xn, c.nx), dy = w.def_dim(yn, c.ny);
  const int xv = w.def_var(xn, nc3::DOUBLE, {dx}), yv = w.def_var(yn, nc3::DOUBLE, {dy});
  m.e = w.def_var("MaxE", nc3::FLOAT, {dy, dx});
  m.v = w.def_var("MaxV", nc3::FLOAT, {dy, dx});
  w.put_att_text(m.e, "name", "Maximal Water Elevation");
  w.put_att_text(m.e, "units", "m");
  w.put_att_text(m.v, "name", "Maximal Current");
  w.put_att_text(m.v, "units", "m/s");
  w.put_att_text(xv, "name", cart ? "x-axis" : "longitude");
  w.put_att_text(xv, "units", cart ? "meters" : "degrees East");
  w.put_att_text(yv, "name", cart ? "y-axis" : "latitude");
  w.put_att_text(yv, "units", cart ? "meters" : "degrees North");
  w.enddef();
  w.put_var(xv, c.x.data(), c.nx);
  w.put_var(yv, c.y.data(), c.ny);
  w.sync();
  return m;
}

struct GageFile {  // opennc4gages.f
  std::unique_ptr<nc3::Writer> w;
  int t = -1, g = -1, u = -1, v = -1;
  int64_t nrec = 0;
};

GageFile open_gages(const std::string& fname, const Case& c) {
  GageFile f;
  f.w.reset(new nc3::Writer(fname));
  nc3::Writer& w = *f.w;
  const bool cart = c.p.cartesian;
  const int dp = w.def_dim("point", c.p.ngages), dt = w.def_dim("time", 0);
  const int xv = w.def_var(cart ? "xxx" : "lon", nc3::DOUBLE, {dp});
  const int yv = w.def_var(cart ? "yyy" : "lat", nc3::DOUBLE, {dp});
  f.t = w.def_var("time", nc3::DOUBLE, {dt});
  f.g = w.def_var("gage", nc3::DOUBLE, {dt, dp});
  if (c.xrun) f.u = w.def_var("u", nc3::DOUBLE, {dt, dp});
  if (c.yrun) f.v = w.def_var("v", nc3::DOUBLE, {dt, dp});
  w.put_att_text(f.g, "name", "wave elevation at the gage");
  w.put_att_text(f.g, "units", "meters");
  if (f.u >= 0) {
    w.put_att_text(f.u, "name", "x (zonal) velocity");
    w.put_att_text(f.u, "units", "m/s");
  }
  if (f.v >= 0) {
    w.put_att_text(f.v, "name", "y (meridional) velocity");
    w.put_att_text(f.v, "units", "m/s");
  }
  w.put_att_text(xv, "name", cart ? "x-axis" : "longitude");
  w.put_att_text(xv, "units", cart ? "meters" : "degrees_east");
  w.put_att_text(yv, "name", cart ? "y-axis" : "latitude");
  w.put_att_text(yv, "units", cart ? "meters" : "degrees_north");
  w.put_att_text(f.t, "name", "time");
  w.put_att_text(f.t, "units", "seconds");
  w.put_att_text(-1, "model", "Cliffs");
  w.enddef();
  std::vector<double> gx(c.p.ngages), gy(c.p.ngages);
  for (int k = 0; k < c.p.ngages; ++k) {
    gx[k] = c.x[c.p.gage_i[k] - 1];
    gy[k] = c.y[c.p.gage_j[k] - 1];
  }
  w.put_var(xv, gx.data(), c.p.ngages);
  w.put_var(yv, gy.data(), c.p.ngages);
  return f;
}

struct FeedFiles {  // opennc4feed.f: the four edges of one child
  std::unique_ptr<nc3::Writer> w[4];
  int64_t nrec = 0;
};

FeedFiles open_feed(const std::string& base, int mm, int nn) {
  FeedFiles f;
  static const char* side[] = {"west", "east", "south", "north"};
  for (int s = 0; s < 4; ++s) {
    f.w[s].reset(new nc3::Writer(base + "_" + side[s] + ".nc"));
    nc3::Writer& w = *f.w[s];
    const int dp = w.def_dim("pnt", s < 2 ? nn : mm), du = w.def_dim("uvq", 3), dt = w.def_dim("tim", 0);
    w.def_var("vals", nc3::DOUBLE, {dt, du, dp});
    w.def_var("time", nc3::DOUBLE, {dt});
    w.enddef();
  }
  return f;
}

// ---- the run ------------------------------------------------------------------

struct Outputs {
  std::vector<SeaFile> sea;  // h, then u if xrun, then v if yrun
  std::vector<int> sea_who;
  int nxsub = 0, nysub = 0;
  int64_t ishot = 0;
  MaxFile max;
  std::unique_ptr<GageFile> gages;
  std::vector<FeedFiles> feeds;
};

Outputs open_outputs(const Case& c, const std::string& casename, const std::string& outprefix, Log& log) {
  Outputs o;
  for (const auto& n : c.nests) o.feeds.push_back(open_feed(outprefix + "_" + n.name, n.mm, n.nn));
  o.max = open_max(casename + "_maxwave.nc", c);
  log.line("Maxwave output to: " + casename + "_maxwave.nc");
  if (c.p.seaout <= c.p.steps_total) {
    o.nxsub = (c.nx - 1) / c.p.lonsub + 1;
    o.nysub = (c.ny - 1) / c.p.latsub + 1;
    std::vector<double> lon, lat;
    for (int i = 0; i < c.nx; i += c.p.lonsub) lon.push_back(c.x[i]);
    for (int j = 0; j < c.ny; j += c.p.latsub) lat.push_back(c.y[j]);
    o.sea.push_back(open_sea(casename + "_sea_h.nc", 1, lon, lat, c.p.cartesian));
    o.sea_who.push_back(1);
    if (c.xrun) {
      o.sea.push_back(open_sea(casename + "_sea_u.nc", 2, lon, lat, c.p.cartesian));
      o.sea_who.push_back(2);
    }
    if (c.yrun) {
      o.sea.push_back(open_sea(casename + "_sea_v.nc", 3, lon, lat, c.p.cartesian));
      o.sea_who.push_back(3);
    }
    log.line("Screenshot output to: " + casename + "_sea_h.nc");
  }
  if (c.p.ngages >= 1) {
    o.gages.reset(new GageFile(open_gages(casename + "_gages.nc", c)));
    log.line("Time-series output to  " + casename + "_gages.nc");
  }
  return o;
}

void write_sea(Outputs& o, const float* h, const float* u, const float* v, double t, Log& log) {
  const int64_t n = (int64_t)o.nxsub * o.nysub;
  float mx = kNan;
  for (int64_t k = 0; k < n; ++k) mx = std::max(mx, h[k]);
  for (size_t s = 0; s < o.sea.size(); ++s) {
    const float* f = o.sea_who[s] == 1 ? h : o.sea_who[s] == 2 ? u : v;
    o.sea[s].w->put_record(o.sea[s].tvar, o.ishot, &t, 1);
    o.sea[s].w->put_record(o.sea[s].var, o.ishot, f, n);
    o.sea[s].w->sync();
  }
  ++o.ishot;
  std::ostringstream m;
  m << "screenshot " << o.ishot << " at " << t << " sec; Max elevation " << mx;
  log.line(m.str());
}

void write_gage_record(GageFile& g, int ng, const double* e, const double* u, const double* v, double t) {
  g.w->put_record(g.t, g.nrec, &t, 1);
  g.w->put_record(g.g, g.nrec, e, ng);
  if (g.u >= 0) g.w->put_record(g.u, g.nrec, u, ng);
  if (g.v >= 0) g.w->put_record(g.v, g.nrec, v, ng);
  g.w->sync();
  g.nrec++;
}

void write_max(Outputs& o, const float* e, const float* v, int64_t n) {
  std::vector<double> de(e, e + n), dv(v, v + n);
  o.max.w->put_var(o.max.e, de.data(), n);
  o.max.w->put_var(o.max.v, dv.data(), n);
  o.max.w->sync();
}

void write_feed(FeedFiles& f, const double* w, const double* e, const double* s, const double* n, int mm, int nn,
                double t) {
  const double* parts[4] = {w, e, s, n};
  for (int k = 0; k < 4; ++k) {
    const int len = k < 2 ? nn : mm;
    f.w[k]->put_record(1, f.nrec, &t, 1);
    f.w[k]->put_record(0, f.nrec, parts[k], 3 * (int64_t)len);
    f.w[k]->sync();
  }
  f.nrec++;
}

// --dry-run: a JSON summary and the initial records computed on the host
int dry_run(const Case& c, const std::string& casename, const std::string& outprefix, Log& log) {
  Outputs o = open_outputs(c, casename, outprefix, log);
  const double ground = c.p.ground;
  if (!o.sea.empty()) {
    const size_t n = (size_t)o.nxsub * o.nysub;
    std::vector<float> h(n), u(n), v(n);
    size_t k = 0;
    for (int j = 0; j < c.ny; j += c.p.latsub)
      for (int i = 0; i < c.nx; i += c.p.lonsub, ++k) {
        const size_t q = (size_t)j * c.nx + i;
        const bool wet = c.H[q] > ground;
        h[k] = wet ? (float)(c.H[q] - c.dep[q]) : kNan;
        u[k] = wet ? (float)c.u[q] : kNan;
        v[k] = wet ? (float)c.v[q] : kNan;
      }
    write_sea(o, h.data(), u.data(), v.data(), c.t0, log);
  }
  if (o.gages) {
    const int ng = c.p.ngages;
    std::vector<double> e(ng), u(ng), v(ng);
    for (int k = 0; k < ng; ++k) {
      const size_t q = (size_t)(c.p.gage_j[k] - 1) * c.nx + (c.p.gage_i[k] - 1);
      e[k] = c.H[q] > ground ? c.H[q] - c.dep[q] : (double)kNan;
      u[k] = c.u[q];
      v[k] = c.v[q];
    }
    write_gage_record(*o.gages, ng, e.data(), u.data(), v.data(), c.t0);
  }
  double hmax = -1e300, depmin = 1e300, depmax = -1e300, esum = 0;
  for (size_t q = 0; q < c.dep.size(); ++q) {
    depmin = std::min(depmin, c.dep[q]);
    depmax = std::max(depmax, c.dep[q]);
    if (c.H[q] > ground) {
      hmax = std::max(hmax, c.H[q] - c.dep[q]);
      esum += c.H[q] - c.dep[q];
    }
  }
  std::printf("{\"nx\": %d, \"ny\": %d, \"cartesian\": %s, \"nests\": %d, \"children\": [", c.nx, c.ny,
              c.p.cartesian ? "true" : "false", c.p.nests);
  for (size_t k = 0; k < c.nests.size(); ++k)
    std::printf("%s{\"name\": \"%s\", \"mm\": %d, \"nn\": %d, \"W_nx\": %d, \"E_nx\": %d, \"S_ny\": %d, "
                "\"N_ny\": %d}",
                k ? ", " : "", c.nests[k].name.c_str(), c.nests[k].mm, c.nests[k].nn, c.nests[k].W_nx,
                c.nests[k].E_nx, c.nests[k].S_ny, c.nests[k].N_ny);
  std::printf("], \"cuke\": %.17g, \"ground\": %.17g, \"crough\": %.17g, \"itopo\": %d, \"dwall\": %.17g, "
              "\"dt\": %.17g, \"steps_total\": %d, \"quake\": %d, \"freeze\": %s, \"seaout\": %d, "
              "\"lonsub\": %d, \"latsub\": %d, \"bndout\": %d, \"maxout\": %d, \"ngages\": %d, \"gout\": %d, ",
              c.p.cuke, c.p.ground, c.p.crough, c.p.itopo, c.p.dwall, c.p.dt, c.p.steps_total, c.p.quake,
              c.p.freeze ? "true" : "false", c.p.seaout, c.p.lonsub, c.p.latsub, c.p.bndout, c.p.maxout,
              c.p.ngages, c.p.gout);
  std::printf("\"bndr_input\": %s, \"nt\": %d, \"irec\": %d, \"t0\": %.17g, \"hinput\": %s, \"uinput\": %s, "
              "\"vinput\": %s, \"tsrc\": %.17g, \"dep_min\": %.17g, \"dep_max\": %.17g, \"eta_max\": %.17g, "
              "\"eta_sum\": %.17g, \"has_zeta\": %s, \"master\": \"%s\"}\n",
              c.bndr_input ? "true" : "false", c.nt, c.irec, c.t0, c.hinput ? "true" : "false",
              c.uinput ? "true" : "false", c.vinput ? "true" : "false", c.tsrc_used, depmin, depmax, hmax, esum,
              c.has_zeta ? "true" : "false", c.p.master_name.c_str());
  return 0;
}

int run(const Case& c, const std::string& casename, const std::string& outprefix, Log& log) {
  const int nx = c.nx, ny = c.ny;
  const int64_t cells = (int64_t)nx * ny;
  // MasterGrid.f:85-121 through the library
  std::vector<double> dx(std::max(nx - 1, 1)), rs(ny, 1.0), dy(std::max(ny - 1, 1)), zeta(ny, 0.0);
  check(cliffs_gpu_metrics(nx, ny, c.p.cartesian ? 1 : 0, c.x.data(), c.y.data(), dx.data(), rs.data(), dy.data(),
                           zeta.data()),
        "metrics");
  if (c.has_zeta) zeta = c.zeta;
  cliffs_grid_desc d{};
  d.nx = nx;
  d.ny = ny;
  d.dep = c.dep.data();
  d.dx = c.xrun ? dx.data() : nullptr;
  d.row_scale = (c.xrun && !c.p.cartesian) ? rs.data() : nullptr;
  d.dy = c.yrun ? dy.data() : nullptr;
  d.zeta = c.yrun ? zeta.data() : nullptr;
  d.ground = c.p.ground;
  d.crough = c.p.crough;
  d.dt = c.p.dt;
  cliffs_ctx* ctx = nullptr;
  check(cliffs_gpu_create(&d, &ctx), "create");
  struct Guard {
    cliffs_ctx* c;
    ~Guard() { cliffs_gpu_destroy(c); }
  } guard{ctx};
  check(cliffs_gpu_set_initial(ctx, c.H.data(), c.u.data(), c.v.data()), "set_initial");
  if (c.bndr_input)
    check(cliffs_gpu_set_feed(ctx, c.nt, c.tinput.data(), c.xrun ? c.west.data() : nullptr,
                              c.xrun ? c.east.data() : nullptr, c.yrun ? c.south.data() : nullptr,
                              c.yrun ? c.north.data() : nullptr, c.irec, c.p.freeze ? 1 : 0),
          "set_feed");
  std::vector<int32_t> nest_id;
  for (const auto& n : c.nests) {
    cliffs_nest_desc nd{};
    nd.mm = n.mm;
    nd.nn = n.nn;
    nd.W_nx = n.W_nx;
    nd.E_nx = n.E_nx;
    nd.S_ny = n.S_ny;
    nd.N_ny = n.N_ny;
    nd.W_cx = n.W_cx;
    nd.E_cx = n.E_cx;
    nd.S_cy = n.S_cy;
    nd.N_cy = n.N_cy;
    nd.WE_ny = n.WE_ny.data();
    nd.WE_cy = n.WE_cy.data();
    nd.SN_nx = n.SN_nx.data();
    nd.SN_cx = n.SN_cx.data();
    int32_t id = -1;
    check(cliffs_gpu_nest_add(ctx, &nd, &id), "nest_add");
    nest_id.push_back(id);
  }
  Outputs o = open_outputs(c, casename, outprefix, log);
  double t = c.t0;
  const int ng = c.p.ngages;
  std::vector<float> me(cells), mv(cells);
  auto maxwave = [&]() {
    check(cliffs_gpu_get_maxwave(ctx, me.data(), mv.data()), "maxwave");
    write_max(o, me.data(), mv.data(), cells);
  };
  // Screenshots, gauge records and child feed records are asynchronous
  // outputs: queued on the device in order with the steps, copied to pinned
  // host slots behind them, and written to their files once the copy has
  // landed.  The loop runs up to kDepth records of a kind ahead of the files;
  // a kind whose slots are all in flight writes its oldest record first.
  constexpr int kDepth = 3;
  enum Kind { kSea = 0, kGage = 1, kFeed = 2 };
  struct Pending {
    int64_t ticket;
    double t;
    int kind, child, slot;
  };
  std::deque<Pending> queue;
  std::vector<void*> pinned;
  auto host = [&](size_t bytes) {
    void* p = nullptr;
    check(cliffs_gpu_host_alloc((int64_t)std::max<size_t>(bytes, 8), &p), "host_alloc");
    pinned.push_back(p);
    return p;
  };
  struct PinnedGuard {
    std::vector<void*>& v;
    ~PinnedGuard() {
      for (void* p : v) cliffs_gpu_host_free(p);
    }
  } pinned_guard{pinned};
  const size_t nsub = (size_t)o.nxsub * o.nysub;
  float* sea_buf = o.sea.empty() ? nullptr : (float*)host(kDepth * 3 * nsub * sizeof(float));
  double* gage_buf = ng >= 1 ? (double*)host(kDepth * 3 * (size_t)ng * sizeof(double)) : nullptr;
  std::vector<double*> feed_buf;
  std::vector<int32_t*> feed_arr;
  for (const auto& n : c.nests) {
    feed_buf.push_back((double*)host(kDepth * 6 * (size_t)(n.mm + n.nn) * sizeof(double)));
    feed_arr.push_back((int32_t*)host(kDepth * sizeof(int32_t)));
  }
  std::vector<int> in_flight(2 + c.nests.size(), 0), next_slot(2 + c.nests.size(), 0);
  std::vector<int32_t> arrived(c.nests.size(), 0);
  auto write_front = [&]() {
    const Pending p = queue.front();
    queue.pop_front();
    check(cliffs_gpu_output_wait(ctx, p.ticket), "output_wait");
    if (p.kind == kSea) {
      const float* b = sea_buf + (size_t)p.slot * 3 * nsub;
      write_sea(o, b, b + nsub, b + 2 * nsub, p.t, log);
    } else if (p.kind == kGage) {
      const double* b = gage_buf + (size_t)p.slot * 3 * ng;
      write_gage_record(*o.gages, ng, b, b + ng, b + 2 * ng, p.t);
    } else {
      const int k = p.child, mm = c.nests[k].mm, nn = c.nests[k].nn;
      if (feed_arr[k][p.slot]) {  // feed_children_grid.f: a record once the wave is in the footprint
        if (!arrived[k]) {
          arrived[k] = 1;
          std::ostringstream m;
          m << "reached child grid " << k + 1 << " at " << p.t << "sec";
          log.line(m.str());
        }
        const double* b = feed_buf[k] + (size_t)p.slot * 6 * (mm + nn);
        write_feed(o.feeds[k], b, b + 3 * (size_t)nn, b + 6 * (size_t)nn, b + 6 * (size_t)nn + 3 * (size_t)mm,
                   mm, nn, p.t);
      }
    }
    --in_flight[p.kind == kFeed ? 2 + p.child : p.kind];
  };
  // a free slot of kind index q: the oldest records are written until one is
  auto slot_for = [&](int q) {
    while (in_flight[q] >= kDepth) write_front();
    ++in_flight[q];
    const int s = next_slot[q];
    next_slot[q] = (s + 1) % kDepth;
    return s;
  };
  auto sea = [&]() {
    const int s = slot_for(kSea);
    float* b = sea_buf + (size_t)s * 3 * nsub;
    int64_t tk = 0;
    check(cliffs_gpu_get_sea_state_async(ctx, c.p.lonsub, c.p.latsub, b, b + nsub, b + 2 * nsub, &tk),
          "sea_state");
    queue.push_back({tk, t, kSea, 0, s});
  };
  auto gages = [&]() {
    const int s = slot_for(kGage);
    double* b = gage_buf + (size_t)s * 3 * ng;
    int64_t tk = 0;
    check(cliffs_gpu_get_gauges_async(ctx, ng, c.p.gage_i.data(), c.p.gage_j.data(), b, b + ng, b + 2 * ng, &tk),
          "gauges");
    queue.push_back({tk, t, kGage, 0, s});
  };
  auto feed = [&]() {  // feed_children_grid.f
    for (size_t k = 0; k < c.nests.size(); ++k) {
      const int s = slot_for(2 + (int)k);
      const int mm = c.nests[k].mm, nn = c.nests[k].nn;
      double* b = feed_buf[k] + (size_t)s * 6 * (mm + nn);
      int64_t tk = 0;
      check(cliffs_gpu_feed_child_async(ctx, nest_id[k], c.p.cuke, feed_arr[k] + s, b, b + 3 * (size_t)nn,
                                        b + 6 * (size_t)nn, b + 6 * (size_t)nn + 3 * (size_t)mm, &tk),
            "feed_child");
      queue.push_back({tk, t, kFeed, (int)k, s});
    }
  };
  auto status = [&](int istep) {
    uint32_t flags = 0;
    const int st = cliffs_gpu_status(ctx, &flags);
    if (st == CLIFFS_ERR_NAN || (flags & CLIFFS_ST_NAN))
      throw std::runtime_error("non-finite state by step " + std::to_string(istep));
    check(st, "status");
  };
  // cliffs_main.f:255-297: the initial screenshot, gauge record and child feed
  if (!o.sea.empty()) sea();
  if (ng >= 1) gages();
  if (!c.nests.empty()) feed();
  // cliffs_main.f:300-378: advance to the next output event, then output
  const int total = c.p.steps_total;
  auto next_event = [&](int istep) {
    int nxt = total;
    auto consider = [&](int every, bool on) {
      if (on && every > 0) nxt = std::min(nxt, (istep / every + 1) * every);
    };
    consider(c.p.seaout, !o.sea.empty());
    consider(c.p.gout, ng >= 1);
    consider(c.p.maxout, true);
    consider(c.p.bndout, !c.nests.empty());
    return nxt;
  };
  int istep = 0;
  const auto t_start = std::chrono::steady_clock::now();
  while (istep < total) {
    const int nxt = next_event(istep);
    int32_t done = 0;
    const int r = cliffs_gpu_step(ctx, nxt - istep, &t, &done);
    check(r, "step");
    istep += done;
    if (r == CLIFFS_FEED_ENDED) {
      log.line("bndr feed ended at step " + std::to_string(istep + 1));
      break;
    }
    if (!c.nests.empty() && istep % c.p.bndout == 0) feed();
    if (!o.sea.empty() && istep % c.p.seaout == 0) sea();
    if (ng >= 1 && istep % c.p.gout == 0) gages();
    if (istep % c.p.maxout == 0) {  // synchronises: the status word is read here
      status(istep);
      maxwave();
    }
  }
  while (!queue.empty()) write_front();
  status(istep);
  maxwave();  // cliffs_main.f:380
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  std::ostringstream m;
  m << "time loop: " << istep << " steps in " << secs << " s, "
    << (secs > 0 ? (double)cells * istep / secs / 1e6 : 0.0) << " Mcell-updates/s";
  log.line(m.str());
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  bool dry = false;
  std::vector<std::string> a;
  for (int i = 1; i < argc; ++i) {
    if (std::strcmp(argv[i], "--dry-run") == 0)
      dry = true;
    else
      a.push_back(argv[i]);
  }
  if (a.size() < 5) {
    std::printf("Help: cliffs_gb300 <output dir/prefix> <source dir/> <boundary prefix, 0 for no input> "
                "<area prefix, 0 for no input> <param dir/param file> [<short notes>] [--dry-run]\n");
    return 2;
  }
  auto split = [](const std::string& s, std::string& dir, std::string& name) {
    const size_t k = s.rfind('/');
    dir = k == std::string::npos ? "" : s.substr(0, k + 1);
    name = k == std::string::npos ? s : s.substr(k + 1);
  };
  std::string outdir, casetitle, paramdir, paramfile;
  split(a[0], outdir, casetitle);
  split(a[4], paramdir, paramfile);
  const std::string srcdir = a[1], bprfx = a[2], aprfx = a[3];
  std::string notes;
  for (size_t i = 5; i < a.size(); ++i) notes += a[i] + " ";
  const std::string casename = outdir + casetitle;
  Log log(casename + "_log.txt");
  if (!log.ok()) {
    std::fprintf(stderr, "cannot write %s_log.txt\n", casename.c_str());
    return 1;
  }
  log << stamp() << '\n';
  log.line(notes);
  log.line("Case Title: " + casetitle);
  log.line("Input Data: " + bprfx + ", " + aprfx);
  try {
    Case c = cliffs_host::read_case(srcdir, bprfx, aprfx, paramdir, paramfile);
    for (const std::string& s : c.log) log.line(s);
    const int rc = dry ? dry_run(c, casename, casename, log) : run(c, casename, casename, log);
    log << stamp() << '\n';
    return rc;
  } catch (const std::exception& e) {
    log.line(std::string("error: ") + e.what());
    std::fprintf(stderr, "cliffs_gb300: %s\n", e.what());
    return 1;
  }
}
