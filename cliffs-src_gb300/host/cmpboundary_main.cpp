// cmpboundary_main.cpp -- ComputeBoundaryInput (cmpboundary/cmpboundary.f)
// with its scan and edge interpolation on the GPU (cliffs_boundary_scan,
// cliffs_boundary_edges, include/cliffs_gpu.h).
//
//   cmpboundary_gb300 <full path to h-file> <full path to target grid> <output dir/casetitle> <units (m/cm)>
//
// As the reference (cmpboundary.f:44-190):
// - The still-sea threshold cuke is read from standard input.
// - The target grid's coordinates are its variables on its first and second
//   dimension.  The sea-state files (h, and u and v named by replacing the
//   last 'h' of the path) have dimensions and coordinate variables named
//   tim/TIM, xxx/lon/LON and yyy/lat/LAT; their last variable is the field.
// - Values below -1e10 are missing and count as 0; with units other than m,
//   values are taken as centimetres (times 0.01).
// - The target must lie within the source lattice.  The records start at
//   the first record whose footprint (the lattice cells around the target)
//   holds a value above cuke in magnitude.
// - The output is <casetitle>_<grid name>_{west,east,south,north}.nc: vals
//   (pnt, uvq, tim) and time (tim), as opennc4feed.f defines them.
// The footprint is cut on the host one record at a time, so memory follows
// the footprint, not the source lattice.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/cliffs_gpu.h"
#include "nc3.hpp"

namespace {

bool prefix(const std::string& s, std::initializer_list<const char*> ps) {
  for (const char* p : ps)
    if (s.compare(0, 3, p) == 0) return true;
  return false;
}

// NestedGrid.f:129-148 (cmpboundary.f's copy): the 1-based ip with
// xx(ip) <= xp <= xx(ip+1), and the weight of xx(ip).
void pinpoint(const std::vector<double>& xx, double xp, int32_t* ip_out, double* cp) {
  const int n = (int)xx.size();
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

// The sea-state lattice (ReadSeaLattice.f): coordinates, times, the field.
struct Sea {
  std::vector<double> x, y, t;
  int field = -1;   // the last variable
  int ix = -1, iy = -1, it = -1;  // positions of x, y, time among the field's dims (C order)
};

Sea read_sea(const nc3::Reader& f) {
  Sea s;
  int tv = -1, xv = -1, yv = -1;
  for (int v = 0; v < f.nvars(); ++v) {
    const std::string& n = f.var(v).name;
    if (prefix(n, {"tim", "TIM"})) tv = v;
    else if (prefix(n, {"xxx", "LON", "lon"})) xv = v;
    else if (prefix(n, {"yyy", "LAT", "lat"})) yv = v;
  }
  if (tv < 0 || xv < 0 || yv < 0) throw nc3::Error("sea state file without time, x or y variable");
  s.x = f.get_double(xv);
  s.y = f.get_double(yv);
  s.t = f.get_double(tv);
  s.field = f.nvars() - 1;
  const std::vector<int32_t>& d = f.var(s.field).dims;
  if (d.size() != 3) throw nc3::Error("sea state field is not 3-D");
  for (int k = 0; k < 3; ++k) {
    const std::string& n = f.dim(d[k]).name;
    if (prefix(n, {"tim", "TIM"})) s.it = k;
    else if (prefix(n, {"xxx", "LON", "lon"})) s.ix = k;
    else if (prefix(n, {"yyy", "LAT", "lat"})) s.iy = k;
  }
  if (s.it != 0 || s.iy != 1 || s.ix != 2) throw nc3::Error("sea state field is not (time, y, x)");
  return s;
}

// The footprint cube: lattice columns ix1..ix1+nx-1, rows iy1..iy1+ny-1
// (1-based), records rec0..rec0+nt-1 (0-based), x fastest, as float.
std::vector<float> footprint(const nc3::Reader& f, const Sea& s, int ix1, int iy1, int nx, int ny, int rec0, int nt) {
  const size_t NX = s.x.size(), NY = s.y.size();
  std::vector<float> c((size_t)nx * ny * nt);
  const bool rec = f.var(s.field).is_record;
  const std::vector<double> all = rec ? std::vector<double>() : f.get_double(s.field);  // a fixed time dimension
  for (int k = 0; k < nt; ++k) {
    const std::vector<double> one = rec ? f.get_records_double(s.field, rec0 + k, 1) : std::vector<double>();
    const double* r = rec ? one.data() : all.data() + (size_t)(rec0 + k) * NX * NY;
    if (rec && one.size() != NX * NY) throw nc3::Error("sea state record is not nx x ny");
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        c[(size_t)k * nx * ny + (size_t)j * nx + i] = (float)r[(size_t)(iy1 - 1 + j) * NX + (ix1 - 1 + i)];
  }
  return c;
}

void check(int r, const char* what) {
  if (r) throw nc3::Error(std::string(what) + ": " + cliffs_gpu_strerror(r));
}

// opennc4feed.f and output_bndr.f: one edge's file
void write_edge(const std::string& path, int npnt, const std::vector<double>& vals, const std::vector<double>& tim) {
  nc3::Writer w(path);
  const int pnt = w.def_dim("pnt", npnt), uvq = w.def_dim("uvq", 3), tm = w.def_dim("tim", 0);
  const int vv = w.def_var("vals", nc3::DOUBLE, {tm, uvq, pnt});
  const int vt = w.def_var("time", nc3::DOUBLE, {tm});
  w.enddef();
  for (size_t k = 0; k < tim.size(); ++k) {
    w.put_record(vv, (int64_t)k, vals.data() + k * 3 * npnt, 3 * (int64_t)npnt);
    w.put_record(vt, (int64_t)k, &tim[k], 1);
  }
  w.close();
}

}  // namespace

namespace {

int run(int argc, char** argv) {
  if (argc != 5) {
    std::printf(" Help: */ComputeBoundaryInput <full path to h-file> <full path to target grid> "
                "<output dir/casetitle> <units(m/cm)>\n");
    return 0;
  }
  std::string pathin = argv[1];
  const std::string grid = argv[2], casetitle = argv[3], units = argv[4];
  const double scale = units == "m" ? 1.0 : 0.01;
  std::printf(" Still sea threshold (m) ? \n");
  double cuke = 0;
  if (!(std::cin >> cuke)) throw nc3::Error("no still sea threshold on standard input");
  std::printf(" Still sea threshold (m): %g\n", cuke);
  // the target grid (ReadGridLattice.f): its coordinate vectors
  std::printf(" Target area bathy/topo file:  %s\n", grid.c_str());
  nc3::Reader g(grid);
  if (g.ndims() < 2) throw nc3::Error("target grid with fewer than 2 dimensions");
  int gx = -1, gy = -1;
  for (int v = 0; v < g.nvars(); ++v) {
    const std::vector<int32_t>& d = g.var(v).dims;
    if (d.size() == 1 && d[0] == 0 && gx < 0) gx = v;
    if (d.size() == 1 && d[0] == 1 && gy < 0) gy = v;
  }
  if (gx < 0 || gy < 0) throw nc3::Error("target grid without x and y vectors");
  const std::vector<double> xn = g.get_double(gx), yn = g.get_double(gy);
  const int mm = (int)xn.size(), nn = (int)yn.size();
  std::printf(" grid size %d %d\n", mm, nn);
  // the source lattice (ReadSeaLattice.f)
  std::printf(" Sea state file:  %s\n", pathin.c_str());
  Sea sea;
  {
    nc3::Reader h(pathin);
    sea = read_sea(h);
  }
  const int NX = (int)sea.x.size(), NY = (int)sea.y.size(), NT = (int)sea.t.size();
  std::printf(" Nodes in Sea State Dataset (lon/lat/time): %d %d %d\n", NX, NY, NT);
  if (NX < 2 || NY < 2 || NT < 1) throw nc3::Error("sea state lattice smaller than 2 x 2 x 1");
  std::printf("  Longitude: %g  to %g\n", sea.x.front(), sea.x.back());
  std::printf("   Latitude: %g  to %g\n", sea.y.front(), sea.y.back());
  std::printf("       Time: %g  to %g\n", sea.t.front(), sea.t.back());
  if (xn.front() < sea.x.front() || xn.back() > sea.x.back() || yn.front() < sea.y.front() ||
      yn.back() > sea.y.back()) {
    std::printf(" Target area lon/lat limits: %g %g %g %g\n", xn.front(), xn.back(), yn.front(), yn.back());
    std::printf(" not within source grid limits\n");
    return 1;
  }
  // the target's edges in the source lattice (cmpboundary.f:110-124)
  cliffs_nest_desc t{};
  t.mm = mm;
  t.nn = nn;
  std::vector<int32_t> we(nn), sn(mm);
  std::vector<double> wc(nn), sc(mm);
  pinpoint(sea.y, yn.front(), &t.S_ny, &t.S_cy);
  pinpoint(sea.y, yn.back(), &t.N_ny, &t.N_cy);
  for (int i = 0; i < mm; ++i) pinpoint(sea.x, xn[i], &sn[i], &sc[i]);
  pinpoint(sea.x, xn.front(), &t.W_nx, &t.W_cx);
  pinpoint(sea.x, xn.back(), &t.E_nx, &t.E_cx);
  for (int i = 0; i < nn; ++i) pinpoint(sea.y, yn[i], &we[i], &wc[i]);
  t.WE_ny = we.data();
  t.WE_cy = wc.data();
  t.SN_nx = sn.data();
  t.SN_cx = sc.data();
  // the footprint, and the first record with a signal (scan4wave.f)
  const int ix1 = t.W_nx, iy1 = t.S_ny, nx = t.E_nx + 1 - ix1 + 1, ny = t.N_ny + 1 - iy1 + 1;
  int32_t first = -1;
  {
    nc3::Reader h(pathin);
    const std::vector<float> cube = footprint(h, sea, ix1, iy1, nx, ny, 0, NT);
    check(cliffs_boundary_scan(nx, ny, NT, cube.data(), cuke, &first), "boundary_scan");
  }
  // scan4wave.f reports a first signal at the last record, or none, as no
  // signal; cmpboundary.f carries on all the same with the records from there
  // on (one, or none)
  if (first >= NT)
    std::printf(" no signal above treshold\n");
  else
    std::printf(" signal detected at step %d\n", first);
  const int nnt = NT - first + 1;
  const std::vector<double> tim(sea.t.begin() + (first - 1), sea.t.end());
  // the three fields (get_sea_state.f, InterpolateOntoBndr.f): h, u, v named by the path's last 'h'
  const size_t ic1 = pathin.rfind('/') == std::string::npos ? 0 : pathin.rfind('/') + 1;
  const size_t ic2 = pathin.rfind('h');
  // the reference's test: an 'h' in the file name, neither its first nor its last character
  if (ic2 == std::string::npos || ic2 + 1 >= pathin.size() || ic1 >= ic2) {
    std::printf(" Wrong naming for input dataset\n");
    return 1;
  }
  std::vector<double> w((size_t)3 * nn * nnt), e(w.size()), s((size_t)3 * mm * nnt), n(s.size());
  const char comp[3] = {'h', 'u', 'v'};
  const int ival[3] = {3, 1, 2};
  for (int k = 0; k < 3; ++k) {
    pathin[ic2] = comp[k];
    nc3::Reader h(pathin);
    const Sea sk = read_sea(h);
    if ((int)sk.x.size() != NX || (int)sk.y.size() != NY || (int)sk.t.size() != NT)
      throw nc3::Error(pathin + " does not match the h-file's lattice");
    if (nnt > 0) {
      const std::vector<float> cube = footprint(h, sk, ix1, iy1, nx, ny, first - 1, nnt);
      check(cliffs_boundary_edges(&t, nx, ny, nnt, cube.data(), scale, ival[k], w.data(), e.data(), s.data(),
                                  n.data()),
            "boundary_edges");
    }
    std::printf(" %s is read\n", pathin.c_str());
  }
  // output (opennc4feed.f, output_bndr.f)
  const size_t gs = grid.rfind('/') == std::string::npos ? 0 : grid.rfind('/') + 1;
  const std::string base = casetitle + "_" + grid.substr(gs, grid.size() >= gs + 3 ? grid.size() - 3 - gs : 0);
  write_edge(base + "_west.nc", nn, w, tim);
  write_edge(base + "_east.nc", nn, e, tim);
  write_edge(base + "_south.nc", mm, s, tim);
  write_edge(base + "_north.nc", mm, n, tim);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    return run(argc, argv);
  } catch (const std::exception& ex) {
    std::fprintf(stderr, "cmpboundary_gb300: %s\n", ex.what());
    return 1;
  }
}
