// nc3.hpp -- NetCDF classic format (CDF-1, CDF-2) reader and writer.
//
// The Cliffs driver reads its grids, boundary feed and initial state from
// NetCDF files and writes screenshots, gauges, max-wave fields and child feed
// records to NetCDF files (the nf_* calls of MasterGrid.f, NestedGrid.f,
// get_boundary_feed.f, get_initial_state.f, opennc4*.f and output_*.f).  The
// reference creates them with NF_CLOBBER, i.e. the classic format; this is a
// self-contained implementation of that published format (big-endian header
// of dimensions, attributes and variables, fixed-size variables at their
// offsets, record variables interleaved per record along the unlimited
// dimension).  Variables are addressed in C order: the first dimension of a
// variable is the slowest, so a Fortran array a(nx, ny, nt) is the C array
// [nt][ny][nx].
#pragma once
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace nc3 {

enum Type : int32_t { BYTE = 1, CHAR = 2, SHORT = 3, INT = 4, FLOAT = 5, DOUBLE = 6 };

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct Attr {
  std::string name;
  Type type = CHAR;
  std::vector<uint8_t> raw;  // values as stored (big-endian), unpadded
  std::string text() const { return std::string(raw.begin(), raw.end()); }
};

struct Dim {
  std::string name;
  int64_t len = 0;  // 0 for the unlimited (record) dimension
};

struct Var {
  std::string name;
  std::vector<int32_t> dims;  // dimension ids, slowest first
  std::vector<Attr> atts;
  Type type = DOUBLE;
  int64_t vsize = 0;  // bytes per record (record variable) or in total
  int64_t begin = 0;  // file offset of the data (of record 0)
  bool is_record = false;
};

int type_size(Type t);

// Read access to an existing file.
class Reader {
 public:
  explicit Reader(const std::string& path);
  ~Reader();
  Reader(const Reader&) = delete;
  Reader& operator=(const Reader&) = delete;

  int ndims() const { return (int)dims_.size(); }
  int nvars() const { return (int)vars_.size(); }
  const Dim& dim(int id) const { return dims_.at(id); }
  int64_t dim_len(int id) const;  // the record count for the unlimited dimension
  const Var& var(int id) const { return vars_.at(id); }
  int var_id(const std::string& name) const;  // -1 when absent
  int64_t numrecs() const { return numrecs_; }
  const std::vector<Attr>& global_atts() const { return gatts_; }
  // Number of values of a variable (all records for a record variable).
  int64_t var_count(int id) const;
  // All values of a variable converted to double, in C order.
  std::vector<double> get_double(int id) const;
  // Records [rec0, rec0+nrec) of a record variable (or the whole of a fixed
  // variable when nrec covers it), converted to double.
  std::vector<double> get_records_double(int id, int64_t rec0, int64_t nrec) const;

 private:
  void parse_header();
  void read_at(int64_t off, void* buf, size_t n) const;
  FILE* f_ = nullptr;
  std::string path_;
  int version_ = 1;
  int64_t numrecs_ = 0;
  int64_t recsize_ = 0;
  std::vector<Dim> dims_;
  std::vector<Attr> gatts_;
  std::vector<Var> vars_;
};

// Create a file, define it, then write fixed variables and records.
class Writer {
 public:
  explicit Writer(const std::string& path);
  ~Writer();
  Writer(const Writer&) = delete;
  Writer& operator=(const Writer&) = delete;

  int def_dim(const std::string& name, int64_t len);  // len 0: unlimited
  int def_var(const std::string& name, Type type, const std::vector<int>& dims);
  void put_att_text(int varid, const std::string& name, const std::string& text);  // varid -1: global
  void put_att(int varid, const Attr& a);  // an attribute as read, any type (nf_copy_att)
  void enddef();
  // A fixed variable, all values (C order), converted to the variable's type.
  void put_var(int varid, const double* v, int64_t n);
  // One record of a record variable, converted to the variable's type.
  void put_record(int varid, int64_t rec, const double* v, int64_t n);
  void put_record(int varid, int64_t rec, const float* v, int64_t n);
  // Write the record count into the header and flush (nf_sync).
  void sync();
  void close();

 private:
  void write_at(int64_t off, const void* buf, size_t n);
  void put_converted(int64_t off, Type t, const double* v, const float* fv, int64_t n);
  FILE* f_ = nullptr;
  std::string path_;
  bool defining_ = true;
  int version_ = 1;
  int64_t numrecs_ = 0;
  int64_t recsize_ = 0;
  int64_t header_size_ = 0;
  std::vector<Dim> dims_;
  std::vector<Attr> gatts_;
  std::vector<Var> vars_;
};

}  // namespace nc3
