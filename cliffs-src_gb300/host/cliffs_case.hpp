// cliffs_case.hpp -- one Cliffs run as the reference's driver sets it up.
//
// Reads what cliffs_main.f reads before its time loop, with the same files,
// names and error behaviour:
//   allabout.f          the positional parameter file
//   MasterGrid.f        grid coordinates, depth and the optional width term
//   NestedGrid.f        child grids and their interpolation tables (pinpoint)
//   get_boundary_feed.f <bprfx>_<grid>_{west,east,south,north}.nc and the
//                       first record above the still-sea threshold
//   get_initial_state.f <aprfx>_{h,u,v}.nc at the start time
//   apply_initial_conditions.f, cliffs_main.f:131-137 (wall), 199-216
//                       (deformation of the bottom or the surface)
// The result is what the C ABI takes: depth after wall and deformation, the
// total depth H and velocities before the celerity transform, the feed
// records and the nest tables.  Failures throw CaseError with the message
// the reference writes to its log.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace cliffs_host {

struct CaseError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// allabout.f:20-92
struct Params {
  bool cartesian = true;
  std::string master_path;  // as written in the file (relative to the params dir)
  std::string master_name;  // MBathyFile: base name without directory and ".nc"
  int nests = 0;
  std::vector<std::string> child_paths;  // as written
  std::vector<std::string> child_names;  // ingrids: the path up to ".nc"
  double cuke = 0, ground = 0, crough = 0;
  int itopo = 1;
  double dwall = 0, dt = 0;
  int steps_total = 0, quake = 0;
  bool freeze = true;
  int seaout = 1, lonsub = 1, latsub = 1, bndout = 1, maxout = 1;
  int ngages = 0, gout = 1;
  std::vector<int32_t> gage_i, gage_j;  // 1-based
};

// NestedGrid.f:104-119: left-next parent node and weight per child edge node
struct Nest {
  std::string name;
  int32_t mm = 0, nn = 0;
  std::vector<double> x, y;
  int32_t W_nx = 0, E_nx = 0, S_ny = 0, N_ny = 0;
  double W_cx = 0, E_cx = 0, S_cy = 0, N_cy = 0;
  std::vector<int32_t> WE_ny, SN_nx;
  std::vector<double> WE_cy, SN_cx;
};

struct Case {
  Params p;
  int nx = 0, ny = 0;
  std::vector<double> x, y;
  std::vector<double> dep;   // (ny, nx) C order, after the wall and a bottom deformation
  bool has_zeta = false;
  std::vector<double> zeta;  // MasterGrid.f:118-120: a fourth variable overrides zeta
  bool xrun = false, yrun = false;
  std::vector<Nest> nests;
  // boundary feed
  bool bndr_input = false;
  int nt = 0;
  std::vector<double> tinput;
  std::vector<double> west, east, south, north;  // (nt, 3, len) C order
  int irec = 1;                                  // 1-based start record
  double feed_wave = 0;                          // edge elevation at the start record
  // initial state
  bool hinput = false, uinput = false, vinput = false;
  double t0 = 0;                 // start time tinput(irec)
  double tsrc_used = 0;          // time of the source record applied
  std::vector<double> H, u, v;   // (ny, nx): H = cel before the celerity transform
  std::vector<std::string> log;  // lines the reference writes to its log
};

// pinpoint (NestedGrid.f:129-148): 1-based ip with xx(ip) <= xp <= xx(ip+1)
// by bisection and the weight cp of node ip.
void pinpoint(const double* xx, int n, double xp, int32_t* ip, double* cp);

// apply_initial_conditions.f:7-70: bilinear interpolation of q (nyq, nxq) on
// lattice (xq, yq) added onto p (nyp, nxp) on lattice (xp, yp).
void apply_initial_conditions(int nxq, int nyq, const double* xq, const double* yq, const double* q,
                              int nxp, int nyp, const double* xp, const double* yp, double* p);

// The whole setup of cliffs_main.f:77-227 for the run
//   Cliffs <outdir/prefix> <srcdir/> <bprfx|0> <aprfx|0> <paramdir/paramfile>
Case read_case(const std::string& srcdir, const std::string& bprfx, const std::string& aprfx,
               const std::string& paramdir, const std::string& paramfile);

}  // namespace cliffs_host
