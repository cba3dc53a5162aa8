// nc3.cpp -- NetCDF classic format reader and writer (see nc3.hpp).
#include "nc3.hpp"

#include <cstring>

namespace nc3 {
namespace {

constexpr uint32_t kDimTag = 0x0A, kVarTag = 0x0B, kAttTag = 0x0C;
constexpr double kFillFloat = 9.9692099683868690e+36;  // NC_FILL_FLOAT / NC_FILL_DOUBLE

int64_t pad4(int64_t n) { return (n + 3) & ~int64_t(3); }

uint32_t be32(const uint8_t* p) {
  return (uint32_t(p[0]) << 24) | (uint32_t(p[1]) << 16) | (uint32_t(p[2]) << 8) | uint32_t(p[3]);
}
uint64_t be64(const uint8_t* p) { return (uint64_t(be32(p)) << 32) | be32(p + 4); }
void put32(std::vector<uint8_t>& b, uint32_t v) {
  b.push_back(uint8_t(v >> 24));
  b.push_back(uint8_t(v >> 16));
  b.push_back(uint8_t(v >> 8));
  b.push_back(uint8_t(v));
}
void put64(std::vector<uint8_t>& b, uint64_t v) {
  put32(b, uint32_t(v >> 32));
  put32(b, uint32_t(v));
}
void put_name(std::vector<uint8_t>& b, const std::string& s) {
  put32(b, (uint32_t)s.size());
  b.insert(b.end(), s.begin(), s.end());
  while (b.size() % 4) b.push_back(0);
}

// Value k of a big-endian array of type t, as double.
double value_at(const uint8_t* p, Type t, int64_t k) {
  switch (t) {
    case BYTE: return double(int8_t(p[k]));
    case CHAR: return double(p[k]);
    case SHORT: {
      const uint8_t* q = p + 2 * k;
      return double(int16_t(uint16_t((q[0] << 8) | q[1])));
    }
    case INT: return double(int32_t(be32(p + 4 * k)));
    case FLOAT: {
      const uint32_t u = be32(p + 4 * k);
      float f;
      std::memcpy(&f, &u, 4);
      return double(f);
    }
    case DOUBLE: {
      const uint64_t u = be64(p + 8 * k);
      double d;
      std::memcpy(&d, &u, 8);
      return d;
    }
  }
  throw Error("nc3: unknown type");
}

void store_value(uint8_t* p, Type t, int64_t k, double v) {
  switch (t) {
    case BYTE: p[k] = uint8_t(int8_t(v)); return;
    case CHAR: p[k] = uint8_t(v); return;
    case SHORT: {
      const uint16_t s = uint16_t(int16_t(v));
      p[2 * k] = uint8_t(s >> 8);
      p[2 * k + 1] = uint8_t(s);
      return;
    }
    case INT: {
      const uint32_t u = uint32_t(int32_t(v));
      for (int i = 0; i < 4; ++i) p[4 * k + i] = uint8_t(u >> (24 - 8 * i));
      return;
    }
    case FLOAT: {
      const float f = float(v);
      uint32_t u;
      std::memcpy(&u, &f, 4);
      for (int i = 0; i < 4; ++i) p[4 * k + i] = uint8_t(u >> (24 - 8 * i));
      return;
    }
    case DOUBLE: {
      uint64_t u;
      std::memcpy(&u, &v, 8);
      for (int i = 0; i < 8; ++i) p[8 * k + i] = uint8_t(u >> (56 - 8 * i));
      return;
    }
  }
  throw Error("nc3: unknown type");
}

}  // namespace

int type_size(Type t) {
  switch (t) {
    case BYTE:
    case CHAR: return 1;
    case SHORT: return 2;
    case INT:
    case FLOAT: return 4;
    case DOUBLE: return 8;
  }
  throw Error("nc3: unknown type");
}

// ---------------------------------------------------------------------------
// Reader

Reader::Reader(const std::string& path) : path_(path) {
  f_ = std::fopen(path.c_str(), "rb");
  if (!f_) throw Error("nc3: cannot open " + path);
  try {
    parse_header();
  } catch (...) {
    std::fclose(f_);
    f_ = nullptr;
    throw;
  }
}

Reader::~Reader() {
  if (f_) std::fclose(f_);
}

void Reader::read_at(int64_t off, void* buf, size_t n) const {
  if (std::fseek(f_, (long)off, SEEK_SET) != 0 || std::fread(buf, 1, n, f_) != n)
    throw Error("nc3: short read in " + path_);
}

void Reader::parse_header() {
  std::fseek(f_, 0, SEEK_END);
  const int64_t fsize = std::ftell(f_);
  // the header is at most the whole file; read it in one piece (grids are
  // read afterwards by offset)
  const int64_t hcap = fsize < (1 << 24) ? fsize : (1 << 24);
  std::vector<uint8_t> h((size_t)hcap);
  read_at(0, h.data(), h.size());
  size_t pos = 0;
  auto need = [&](size_t n) {
    if (pos + n > h.size()) throw Error("nc3: truncated header in " + path_);
  };
  auto u32 = [&]() {
    need(4);
    const uint32_t v = be32(&h[pos]);
    pos += 4;
    return v;
  };
  auto name = [&]() {
    const uint32_t n = u32();
    need(n);
    std::string s(reinterpret_cast<const char*>(&h[pos]), n);
    pos += (size_t)pad4(n);
    return s;
  };
  auto attrs = [&](std::vector<Attr>& out) {
    const uint32_t tag = u32(), n = u32();
    if (tag == 0 && n == 0) return;
    if (tag != kAttTag) throw Error("nc3: bad attribute list in " + path_);
    for (uint32_t i = 0; i < n; ++i) {
      Attr a;
      a.name = name();
      a.type = Type(u32());
      const uint32_t cnt = u32();
      const int64_t bytes = int64_t(cnt) * type_size(a.type);
      need((size_t)bytes);
      a.raw.assign(h.begin() + pos, h.begin() + pos + bytes);
      pos += (size_t)pad4(bytes);
      out.push_back(std::move(a));
    }
  };
  need(4);
  if (h[0] != 'C' || h[1] != 'D' || h[2] != 'F' || (h[3] != 1 && h[3] != 2))
    throw Error("nc3: not a NetCDF classic file: " + path_);
  version_ = h[3];
  pos = 4;
  numrecs_ = u32();
  {
    const uint32_t tag = u32(), n = u32();
    if (!(tag == 0 && n == 0)) {
      if (tag != kDimTag) throw Error("nc3: bad dimension list in " + path_);
      for (uint32_t i = 0; i < n; ++i) {
        Dim d;
        d.name = name();
        d.len = u32();
        dims_.push_back(d);
      }
    }
  }
  attrs(gatts_);
  {
    const uint32_t tag = u32(), n = u32();
    if (!(tag == 0 && n == 0)) {
      if (tag != kVarTag) throw Error("nc3: bad variable list in " + path_);
      for (uint32_t i = 0; i < n; ++i) {
        Var v;
        v.name = name();
        const uint32_t nd = u32();
        for (uint32_t k = 0; k < nd; ++k) v.dims.push_back((int32_t)u32());
        attrs(v.atts);
        v.type = Type(u32());
        v.vsize = u32();
        if (version_ == 1) {
          v.begin = u32();
        } else {
          need(8);
          v.begin = (int64_t)be64(&h[pos]);
          pos += 8;
        }
        for (int32_t d : v.dims)
          if (d < 0 || d >= (int32_t)dims_.size()) throw Error("nc3: bad dimension id in " + path_);
        v.is_record = !v.dims.empty() && dims_[v.dims[0]].len == 0;
        vars_.push_back(std::move(v));
      }
    }
  }
  // record size: the per-record slabs of all record variables; a single
  // record variable is not padded
  int nrec = 0;
  int64_t single = 0;
  for (const Var& v : vars_)
    if (v.is_record) {
      ++nrec;
      int64_t n = type_size(v.type);
      for (size_t k = 1; k < v.dims.size(); ++k) n *= dims_[v.dims[k]].len;
      recsize_ += pad4(n);
      single = n;
    }
  if (nrec == 1) recsize_ = single;
}

int64_t Reader::dim_len(int id) const {
  const Dim& d = dims_.at(id);
  return d.len == 0 ? numrecs_ : d.len;
}

int Reader::var_id(const std::string& n) const {
  for (size_t i = 0; i < vars_.size(); ++i)
    if (vars_[i].name == n) return (int)i;
  return -1;
}

int64_t Reader::var_count(int id) const {
  const Var& v = vars_.at(id);
  int64_t n = 1;
  for (size_t k = 0; k < v.dims.size(); ++k) n *= dim_len(v.dims[k]);
  return n;
}

std::vector<double> Reader::get_double(int id) const {
  const Var& v = vars_.at(id);
  if (v.is_record) return get_records_double(id, 0, numrecs_);
  const int64_t n = var_count(id), ts = type_size(v.type);
  std::vector<uint8_t> raw((size_t)(n * ts));
  if (n) read_at(v.begin, raw.data(), raw.size());
  std::vector<double> out((size_t)n);
  for (int64_t k = 0; k < n; ++k) out[(size_t)k] = value_at(raw.data(), v.type, k);
  return out;
}

std::vector<double> Reader::get_records_double(int id, int64_t rec0, int64_t nrec) const {
  const Var& v = vars_.at(id);
  if (!v.is_record) return get_double(id);
  if (rec0 < 0 || rec0 + nrec > numrecs_) throw Error("nc3: record out of range in " + path_);
  int64_t per = 1;
  for (size_t k = 1; k < v.dims.size(); ++k) per *= dims_[v.dims[k]].len;
  const int64_t ts = type_size(v.type);
  std::vector<uint8_t> raw((size_t)(per * ts));
  std::vector<double> out((size_t)(per * nrec));
  for (int64_t r = 0; r < nrec; ++r) {
    if (per) read_at(v.begin + (rec0 + r) * recsize_, raw.data(), raw.size());
    for (int64_t k = 0; k < per; ++k) out[(size_t)(r * per + k)] = value_at(raw.data(), v.type, k);
  }
  return out;
}

// ---------------------------------------------------------------------------
// Writer

Writer::Writer(const std::string& path) : path_(path) {
  f_ = std::fopen(path.c_str(), "w+b");
  if (!f_) throw Error("nc3: cannot create " + path);
}

Writer::~Writer() {
  try {
    close();
  } catch (...) {
  }
}

int Writer::def_dim(const std::string& name, int64_t len) {
  if (!defining_) throw Error("nc3: def_dim after enddef");
  for (const Dim& d : dims_)
    if (len == 0 && d.len == 0) throw Error("nc3: a second unlimited dimension");
  dims_.push_back(Dim{name, len});
  return (int)dims_.size() - 1;
}

int Writer::def_var(const std::string& name, Type type, const std::vector<int>& dims) {
  if (!defining_) throw Error("nc3: def_var after enddef");
  Var v;
  v.name = name;
  v.type = type;
  for (size_t k = 0; k < dims.size(); ++k) {
    if (dims[k] < 0 || dims[k] >= (int)dims_.size()) throw Error("nc3: bad dimension id");
    if (k > 0 && dims_[dims[k]].len == 0) throw Error("nc3: the record dimension must come first");
    v.dims.push_back(dims[k]);
  }
  v.is_record = !v.dims.empty() && dims_[v.dims[0]].len == 0;
  vars_.push_back(std::move(v));
  return (int)vars_.size() - 1;
}

void Writer::put_att_text(int varid, const std::string& name, const std::string& text) {
  if (!defining_) throw Error("nc3: put_att after enddef");
  Attr a;
  a.name = name;
  a.type = CHAR;
  a.raw.assign(text.begin(), text.end());
  (varid < 0 ? gatts_ : vars_.at(varid).atts).push_back(std::move(a));
}

void Writer::put_att(int varid, const Attr& a) {
  if (!defining_) throw Error("nc3: put_att after enddef");
  (varid < 0 ? gatts_ : vars_.at(varid).atts).push_back(a);
}

void Writer::enddef() {
  if (!defining_) return;
  auto header = [&](int version) {
    std::vector<uint8_t> b{'C', 'D', 'F', uint8_t(version)};
    put32(b, (uint32_t)numrecs_);
    auto attlist = [&](const std::vector<Attr>& as) {
      if (as.empty()) {
        put32(b, 0);
        put32(b, 0);
        return;
      }
      put32(b, kAttTag);
      put32(b, (uint32_t)as.size());
      for (const Attr& a : as) {
        put_name(b, a.name);
        put32(b, (uint32_t)a.type);
        put32(b, (uint32_t)(a.raw.size() / type_size(a.type)));
        b.insert(b.end(), a.raw.begin(), a.raw.end());
        while (b.size() % 4) b.push_back(0);
      }
    };
    if (dims_.empty()) {
      put32(b, 0);
      put32(b, 0);
    } else {
      put32(b, kDimTag);
      put32(b, (uint32_t)dims_.size());
      for (const Dim& d : dims_) {
        put_name(b, d.name);
        put32(b, (uint32_t)d.len);
      }
    }
    attlist(gatts_);
    if (vars_.empty()) {
      put32(b, 0);
      put32(b, 0);
    } else {
      put32(b, kVarTag);
      put32(b, (uint32_t)vars_.size());
      for (const Var& v : vars_) {
        put_name(b, v.name);
        put32(b, (uint32_t)v.dims.size());
        for (int32_t d : v.dims) put32(b, (uint32_t)d);
        attlist(v.atts);
        put32(b, (uint32_t)v.type);
        put32(b, (uint32_t)(v.vsize > 0xFFFFFFFCll ? 0xFFFFFFFFu : (uint32_t)v.vsize));
        if (version == 1)
          put32(b, (uint32_t)v.begin);
        else
          put64(b, (uint64_t)v.begin);
      }
    }
    return b;
  };
  // sizes, then offsets (the header length does not depend on the offsets'
  // values, only on the version)
  int nrec = 0;
  int64_t single = 0;
  for (Var& v : vars_) {
    int64_t n = type_size(v.type);
    for (size_t k = v.is_record ? 1 : 0; k < v.dims.size(); ++k) n *= dims_[v.dims[k]].len;
    v.vsize = pad4(n);
    if (v.is_record) {
      ++nrec;
      single = n;
    }
  }
  for (int version = 1; version <= 2; ++version) {
    header_size_ = (int64_t)header(version).size();
    int64_t off = header_size_;
    for (Var& v : vars_)
      if (!v.is_record) {
        v.begin = off;
        off += v.vsize;
      }
    recsize_ = 0;
    for (Var& v : vars_)
      if (v.is_record) {
        v.begin = off + recsize_;
        recsize_ += v.vsize;
      }
    if (nrec == 1) recsize_ = single;
    bool fits = true;
    for (const Var& v : vars_) fits = fits && v.begin <= 0x7FFFFFFFll;
    version_ = version;
    if (fits) break;
  }
  const std::vector<uint8_t> b = header(version_);
  write_at(0, b.data(), b.size());
  defining_ = false;
  // fixed variables start out at the fill value, as in the library's fill mode
  for (const Var& v : vars_)
    if (!v.is_record) {
      const int64_t n = v.vsize / type_size(v.type);
      std::vector<double> fill((size_t)n, kFillFloat);
      if (v.type != FLOAT && v.type != DOUBLE) std::fill(fill.begin(), fill.end(), 0.0);
      put_converted(v.begin, v.type, fill.data(), nullptr, n);
    }
}

void Writer::write_at(int64_t off, const void* buf, size_t n) {
  if (std::fseek(f_, (long)off, SEEK_SET) != 0 || std::fwrite(buf, 1, n, f_) != n)
    throw Error("nc3: write failed on " + path_);
}

void Writer::put_converted(int64_t off, Type t, const double* v, const float* fv, int64_t n) {
  std::vector<uint8_t> raw((size_t)(n * type_size(t)));
  for (int64_t k = 0; k < n; ++k) store_value(raw.data(), t, k, v ? v[k] : double(fv[k]));
  if (!raw.empty()) write_at(off, raw.data(), raw.size());
}

void Writer::put_var(int varid, const double* v, int64_t n) {
  if (defining_) enddef();
  const Var& var = vars_.at(varid);
  if (var.is_record) throw Error("nc3: put_var on a record variable");
  int64_t cnt = 1;
  for (int32_t d : var.dims) cnt *= dims_[d].len;
  if (n != cnt) throw Error("nc3: put_var size mismatch for " + var.name);
  put_converted(var.begin, var.type, v, nullptr, n);
}

void Writer::put_record(int varid, int64_t rec, const double* v, int64_t n) {
  if (defining_) enddef();
  const Var& var = vars_.at(varid);
  if (!var.is_record) throw Error("nc3: put_record on a fixed variable");
  int64_t per = 1;
  for (size_t k = 1; k < var.dims.size(); ++k) per *= dims_[var.dims[k]].len;
  if (n != per) throw Error("nc3: put_record size mismatch for " + var.name);
  put_converted(var.begin + rec * recsize_, var.type, v, nullptr, n);
  if (rec + 1 > numrecs_) numrecs_ = rec + 1;
}

void Writer::put_record(int varid, int64_t rec, const float* v, int64_t n) {
  if (defining_) enddef();
  const Var& var = vars_.at(varid);
  if (!var.is_record) throw Error("nc3: put_record on a fixed variable");
  int64_t per = 1;
  for (size_t k = 1; k < var.dims.size(); ++k) per *= dims_[var.dims[k]].len;
  if (n != per) throw Error("nc3: put_record size mismatch for " + var.name);
  put_converted(var.begin + rec * recsize_, var.type, nullptr, v, n);
  if (rec + 1 > numrecs_) numrecs_ = rec + 1;
}

void Writer::sync() {
  if (!f_) return;
  if (defining_) enddef();
  std::vector<uint8_t> b;
  put32(b, (uint32_t)numrecs_);
  write_at(4, b.data(), 4);
  std::fflush(f_);
}

void Writer::close() {
  if (!f_) return;
  sync();
  std::fclose(f_);
  f_ = nullptr;
}

}  // namespace nc3
