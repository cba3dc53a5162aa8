// depth_ssl_main.cpp -- the depth_ssl tool (depth_ssl/depth_ssl.f) with its
// depth limiter on the GPU (cliffs_depth_ssl, include/cliffs_gpu.h).
//
//   depth_ssl_gb300 <input bathy file> <OutputDir/> <n (0: default params)> [OutputName]
//
// As the reference (depth_ssl.f:38-200):
// - With n = 0 the ratio is alpha = 2 and the minimal flow depth 0.1 m.
//   Otherwise both are asked for on standard input; alpha is clamped to
//   1.5-2.5, and a minimal depth <= 0 is refused.
// - The output is OutputDir/OutputName, or OutputDir/<input name>_ssl.nc.
// - It has the input's first two dimensions, its global attributes and its
//   x, y and depth variables with their attributes.  When the input has more
//   than two dimensions, the 3 x 3 matrix variable comes along on the
//   dimensions Mrow and Mclm.
// - Only the depth changes; it keeps its type (float or double).
// The reference takes the variables by id (1-3, and 4 for the matrix).
// Here they are found by shape: x on the first dimension alone, y on the
// second alone, the depth on both, the matrix on the third and fourth.  On
// the reference's files this picks the same variables, and it also reads
// files whose writer ordered the variables differently.
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/cliffs_gpu.h"
#include "nc3.hpp"

namespace {

// Variable ids by shape (see the header); -1 when absent.
struct Roles {
  int x = -1, y = -1, b = -1, m = -1;
};
Roles find_roles(const nc3::Reader& in) {
  Roles r;
  for (int v = 0; v < in.nvars(); ++v) {
    const std::vector<int32_t>& d = in.var(v).dims;
    if (d.size() == 1 && d[0] == 0 && r.x < 0) r.x = v;
    if (d.size() == 1 && d[0] == 1 && r.y < 0) r.y = v;
    if (d.size() == 2 && d[0] == 1 && d[1] == 0 && r.b < 0) r.b = v;
    if (d.size() == 2 && d[0] == 2 && d[1] == 3 && r.m < 0) r.m = v;
  }
  return r;
}

// The input variable's definition and attributes in the output
// (copy_vardefine, depth_ssl.f:200-219).
int copy_vardefine(const nc3::Reader& in, nc3::Writer& out, int var) {
  const nc3::Var& v = in.var(var);
  std::vector<int> dims(v.dims.begin(), v.dims.end());
  const int id = out.def_var(v.name, v.type, dims);
  for (const nc3::Attr& a : v.atts) out.put_att(id, a);
  return id;
}

int run(int argc, char** argv) {
  if (argc < 4) {
    std::printf(" Help: ./depth_ssl <full path to input bathy file> <OutputDir/> <n (0-default params)> "
                "[OutputName]\n");
    return 0;
  }
  const std::string inname = argv[1], outdir = argv[2], query = argv[3];
  double alpha = 2.0, depmin = 0.1;
  if (query.empty() || query[0] != '0') {
    std::printf(" ssl (1.5 - 2.5)? \n");
    if (!(std::cin >> alpha)) return 1;
    if (alpha < 1.5) alpha = 1.5;
    if (alpha > 2.5) alpha = 2.5;
    std::printf(" minimal flow depth (m)? \n");
    if (!(std::cin >> depmin)) return 1;
    if (depmin <= 0) {
      std::printf(" I do not think so\n");
      return 0;
    }
  }
  std::string outname;
  if (argc > 4) {
    outname = outdir + argv[4];
  } else {
    const size_t slash = inname.rfind('/');
    const size_t b = slash == std::string::npos ? 0 : slash + 1;
    const size_t e = inname.find(".nc", b);
    outname = outdir + inname.substr(b, (e == std::string::npos ? inname.size() : e) - b) + "_ssl.nc";
  }
  std::printf(" processing %s with\n", inname.c_str());
  std::printf(" ssl= %g  min depth= %g\n", alpha, depmin);
  std::printf(" output to %s\n", outname.c_str());

  nc3::Reader in(inname);
  if (in.ndims() < 2) throw nc3::Error("input has fewer than 2 dimensions");
  const Roles R = find_roles(in);
  if (R.x < 0 || R.y < 0 || R.b < 0) throw nc3::Error("input has no x, y and depth variables");
  const int nx = (int)in.dim_len(0), ny = (int)in.dim_len(1);
  nc3::Writer out(outname);
  out.def_dim(in.dim(0).name, nx);
  out.def_dim(in.dim(1).name, ny);
  const bool matrix = in.ndims() > 2;
  if (matrix) {
    out.def_dim("Mrow", 3);
    out.def_dim("Mclm", 3);
  }
  for (const nc3::Attr& a : in.global_atts()) out.put_att(-1, a);
  const int vx = copy_vardefine(in, out, R.x), vy = copy_vardefine(in, out, R.y), vb = copy_vardefine(in, out, R.b);
  const int vm = matrix && R.m >= 0 ? copy_vardefine(in, out, R.m) : -1;
  out.enddef();
  std::printf(" grid size %d %d\n", nx, ny);
  for (int v : {R.x, R.y}) {
    const nc3::Type t = in.var(v).type;
    if (t != nc3::FLOAT && t != nc3::DOUBLE) throw nc3::Error("wrong coordinate type: " + std::to_string((int)t));
  }
  const nc3::Type bt = in.var(R.b).type;
  if (bt != nc3::FLOAT && bt != nc3::DOUBLE) throw nc3::Error("wrong bathy data type: " + std::to_string((int)bt));
  const std::vector<double> x = in.get_double(R.x), y = in.get_double(R.y);
  out.put_var(vx, x.data(), (int64_t)x.size());
  out.put_var(vy, y.data(), (int64_t)y.size());
  std::vector<double> b = in.get_double(R.b);
  if ((int64_t)b.size() != (int64_t)nx * ny) throw nc3::Error("depth is not nx x ny");
  if (bt == nc3::FLOAT)  // a float map is processed in double and stored back as float
    for (double& v : b) v = (double)(float)v;
  int32_t counts[24], status = 0;
  const int r = cliffs_depth_ssl(nx, ny, b.data(), alpha, depmin, counts, &status);
  if (r) throw nc3::Error(std::string("cliffs_depth_ssl: ") + cliffs_gpu_strerror(r));
  for (int phase = 0; phase < 2; ++phase) {
    std::printf(phase == 0 ? " Node-wise depth adjustments in open water:\n" : " Adjustments at coastlines:\n");
    for (int k = 0; k < 12; ++k) {
      std::printf(" passage %d : %d  nodes adjusted\n", k + 1, counts[12 * phase + k]);
      if (counts[12 * phase + k] == 0) break;
    }
    if (status & (1 << phase))
      std::printf(" ATTN: processing is not complete - too rough bathy or too small alpha\n");
  }
  out.put_var(vb, b.data(), (int64_t)b.size());
  if (vm >= 0) {
    if (in.var(R.m).type != nc3::DOUBLE) throw nc3::Error("wrong O2G matrix data type");
    const std::vector<double> m = in.get_double(R.m);
    out.put_var(vm, m.data(), (int64_t)m.size());
  }
  out.close();
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    return run(argc, argv);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "depth_ssl_gb300: %s\n", e.what());
    return 1;
  }
}
