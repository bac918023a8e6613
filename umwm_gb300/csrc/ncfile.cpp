// netCDF classic / 64-bit-offset files without the netCDF library (see
// ncfile.hpp).  Layout, from the published format specification:
//   "CDF" version(1|2), numrecs, dim_list, gatt_list, var_list, data;
//   lists are tag (0x0A dims, 0x0C atts, 0x0B vars) + count, or two zeros;
//   names are length + bytes padded to 4; a variable is name, ndims, dimids,
//   attributes, type, vsize, begin (4 bytes, 8 with version 2); integers and
//   values are big-endian.
#include "ncfile.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>

namespace umwm {
namespace nc {
namespace {

constexpr uint32_t TAG_DIM = 0x0A, TAG_VAR = 0x0B, TAG_ATT = 0x0C;
constexpr uint32_t NC_CHAR = 2, NC_INT = 4, NC_FLOAT = 5;

struct Buf {
  std::vector<unsigned char> b;
  void u32(uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
  }
  void u64(uint64_t v) {
    for (int s = 56; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
  }
  void bytes(const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    b.insert(b.end(), c, c + n);
    while (b.size() % 4) b.push_back(0);
  }
  void name(const std::string& s) {
    u32((uint32_t)s.size());
    bytes(s.data(), s.size());
  }
};

void put_be_floats(const float* in, size_t n, unsigned char* out, bool as_int) {
  for (size_t i = 0; i < n; ++i) {
    uint32_t u;
    if (as_int) {
      const int32_t v = (int32_t)in[i];
      std::memcpy(&u, &v, 4);
    } else {
      std::memcpy(&u, &in[i], 4);
    }
    out[4 * i] = (unsigned char)(u >> 24);
    out[4 * i + 1] = (unsigned char)(u >> 16);
    out[4 * i + 2] = (unsigned char)(u >> 8);
    out[4 * i + 3] = (unsigned char)u;
  }
}

struct FileCloser {
  void operator()(FILE* f) const {
    if (f) std::fclose(f);
  }
};
using File = std::unique_ptr<FILE, FileCloser>;

}  // namespace

bool write(const std::string& path, const std::vector<std::pair<std::string, size_t>>& dims,
           const std::vector<Var>& vars, std::string& err, size_t numrecs) {
  std::vector<size_t> count(vars.size(), 1);  // elements per record (all elements for fixed-size variables)
  std::vector<bool> rec(vars.size(), false);
  int nrecdims = 0;
  for (auto& d : dims) {
    if (d.second == 0) ++nrecdims;
    if (d.second > 0xFFFFFFFFull) {
      err = "netCDF write: dimension length out of range";
      return false;
    }
  }
  if (nrecdims > 1) {
    err = "netCDF write: more than one record dimension";
    return false;
  }
  for (size_t v = 0; v < vars.size(); ++v)
    for (size_t a = 0; a < vars[v].dims.size(); ++a) {
      const int d = vars[v].dims[a];
      if (d < 0 || d >= (int)dims.size()) {
        err = "netCDF write: bad dimension id";
        return false;
      }
      if (dims[d].second == 0) {
        if (a != 0) {
          err = "netCDF write: the record dimension must come first";
          return false;
        }
        rec[v] = true;
      } else {
        count[v] *= dims[d].second;
      }
    }
  bool any_rec = false;
  for (bool r : rec) any_rec = any_rec || r;
  // header with every variable's begin offset; its size does not depend on them
  auto header = [&](const std::vector<uint64_t>& begin) {
    Buf h;
    h.bytes("CDF\x02", 4);
    h.u32(any_rec ? (uint32_t)numrecs : 0u);  // records
    h.u32(TAG_DIM);
    h.u32((uint32_t)dims.size());
    for (auto& d : dims) {
      h.name(d.first);
      h.u32((uint32_t)d.second);
    }
    h.u32(0);  // no global attributes
    h.u32(0);
    h.u32(TAG_VAR);
    h.u32((uint32_t)vars.size());
    for (size_t v = 0; v < vars.size(); ++v) {
      const Var& x = vars[v];
      h.name(x.name);
      h.u32((uint32_t)x.dims.size());
      for (int d : x.dims) h.u32((uint32_t)d);
      if (x.atts.empty()) {
        h.u32(0);
        h.u32(0);
      } else {
        h.u32(TAG_ATT);
        h.u32((uint32_t)x.atts.size());
        for (auto& a : x.atts) {
          h.name(a.first);
          h.u32(NC_CHAR);
          h.u32((uint32_t)a.second.size());
          h.bytes(a.second.data(), a.second.size());
        }
      }
      h.u32(x.is_int ? NC_INT : NC_FLOAT);
      const uint64_t vs = count[v] * 4;
      h.u32(vs > 0xFFFFFFFCull ? 0xFFFFFFFFu : (uint32_t)vs);  // too large: only legal for the last variable
      h.u64(begin[v]);
    }
    return h;
  };
  // data: the fixed-size variables in order, then the records, each the
  // slabs of the record variables in order
  std::vector<size_t> order;
  for (size_t v = 0; v < vars.size(); ++v)
    if (!rec[v]) order.push_back(v);
  for (size_t v = 0; v < vars.size(); ++v)
    if (rec[v]) order.push_back(v);
  // a variable of more than 4 GiB is only legal as the last fixed-size one of a file without records
  for (size_t a = 0; a < order.size(); ++a)
    if (count[order[a]] * 4 > 0xFFFFFFFCull && (any_rec || a + 1 != order.size())) {
      err = "netCDF write: only the last variable may exceed 4 GiB";
      return false;
    }
  std::vector<uint64_t> begin(vars.size(), 0);
  const size_t hsize = header(begin).b.size();
  uint64_t off = hsize;
  for (size_t v : order) {
    begin[v] = off;
    off += (count[v] * 4 + 3) / 4 * 4;
  }
  const Buf h = header(begin);
  File f(std::fopen(path.c_str(), "wb"));
  if (!f) {
    err = "netCDF write: cannot create " + path;
    return false;
  }
  if (std::fwrite(h.b.data(), 1, h.b.size(), f.get()) != h.b.size()) {
    err = "netCDF write: write failed on " + path;
    return false;
  }
  const size_t CH = 1 << 20;
  std::vector<float> vals(CH);
  std::vector<unsigned char> raw(CH * 4);
  // elements [lo, lo + cnt) of variable v
  auto put = [&](size_t v, size_t lo, size_t cnt) {
    for (size_t first = 0; first < cnt; first += CH) {
      const size_t n = std::min(CH, cnt - first);
      if (!vars[v].fill(lo + first, n, vals.data())) {
        err = "netCDF write: no data for variable " + vars[v].name;
        return false;
      }
      put_be_floats(vals.data(), n, raw.data(), vars[v].is_int);
      if (std::fwrite(raw.data(), 1, n * 4, f.get()) != n * 4) {
        err = "netCDF write: write failed on " + path;
        return false;
      }
    }
    return true;
  };
  for (size_t v : order)
    if (!rec[v] && !put(v, 0, count[v])) return false;
  for (size_t r = 0; any_rec && r < numrecs; ++r)
    for (size_t v : order)
      if (rec[v] && !put(v, r * count[v], count[v])) return false;
  if (std::fflush(f.get()) != 0) {
    err = "netCDF write: flush failed on " + path;
    return false;
  }
  return true;
}

namespace {

struct Reader {
  FILE* f;
  bool ok = true;
  uint32_t u32() {
    unsigned char c[4];
    if (std::fread(c, 1, 4, f) != 4) ok = false;
    return ((uint32_t)c[0] << 24) | ((uint32_t)c[1] << 16) | ((uint32_t)c[2] << 8) | c[3];
  }
  uint64_t u64() {
    const uint64_t hi = u32();
    return (hi << 32) | u32();
  }
  void skip(size_t n) {
    if (std::fseek(f, (long)((n + 3) / 4 * 4), SEEK_CUR) != 0) ok = false;
  }
  std::string name() {
    const uint32_t n = u32();
    if (!ok || n > (1u << 20)) {
      ok = false;
      return {};
    }
    std::string s(n, '\0');
    if (n && std::fread(&s[0], 1, n, f) != n) ok = false;
    if ((n % 4) && std::fseek(f, (long)(4 - n % 4), SEEK_CUR) != 0) ok = false;
    return s;
  }
};

size_t type_size(uint32_t t) {
  switch (t) {
    case 1: case 2: return 1;
    case 3: return 2;
    case 4: case 5: return 4;
    case 6: return 8;
    default: return 0;
  }
}

void skip_atts(Reader& r) {
  const uint32_t tag = r.u32(), n = r.u32();
  if (tag == 0) return;
  for (uint32_t a = 0; a < n && r.ok; ++a) {
    r.name();
    const uint32_t t = r.u32(), cnt = r.u32();
    const size_t ts = type_size(t);
    if (!ts) {
      r.ok = false;
      return;
    }
    r.skip((size_t)cnt * ts);
  }
}

}  // namespace

bool read_float(const std::string& path, const std::string& name, std::vector<size_t>& shape,
                std::vector<float>& values, std::string& err) {
  File f(std::fopen(path.c_str(), "rb"));
  if (!f) {
    err = "netCDF read: cannot open " + path;
    return false;
  }
  Reader r{f.get()};
  char magic[4];
  if (std::fread(magic, 1, 4, f.get()) != 4 || std::memcmp(magic, "CDF", 3) != 0 ||
      (magic[3] != 1 && magic[3] != 2)) {
    err = "netCDF read: " + path + " is not a netCDF classic or 64-bit-offset file";
    return false;
  }
  const bool v2 = magic[3] == 2;
  r.u32();  // numrecs
  std::vector<size_t> dimlen;
  uint32_t tag = r.u32(), n = r.u32();
  if (tag == TAG_DIM)
    for (uint32_t d = 0; d < n && r.ok; ++d) {
      r.name();
      dimlen.push_back(r.u32());
    }
  skip_atts(r);  // global attributes
  tag = r.u32();
  n = r.u32();
  for (uint32_t v = 0; v < n && r.ok && tag == TAG_VAR; ++v) {
    const std::string vn = r.name();
    const uint32_t nd = r.u32();
    std::vector<size_t> sh;
    for (uint32_t d = 0; d < nd && r.ok; ++d) {
      const uint32_t id = r.u32();
      if (id >= dimlen.size()) {
        err = "netCDF read: bad dimension id in " + path;
        return false;
      }
      sh.push_back(dimlen[id]);
    }
    skip_atts(r);
    const uint32_t t = r.u32();
    r.u32();  // vsize
    const uint64_t begin = v2 ? r.u64() : r.u32();
    if (!r.ok) break;
    if (vn != name) continue;
    if (t != NC_FLOAT) {
      err = "netCDF read: variable " + name + " is not float";
      return false;
    }
    size_t cnt = 1;
    for (size_t s : sh) cnt *= s;
    for (size_t s : sh)
      if (s == 0) {
        err = "netCDF read: record variables are not supported (" + name + ")";
        return false;
      }
    if (std::fseek(f.get(), (long)begin, SEEK_SET) != 0) {
      err = "netCDF read: seek failed in " + path;
      return false;
    }
    values.resize(cnt);
    std::vector<unsigned char> raw(std::min<size_t>(cnt, 1 << 20) * 4);
    for (size_t first = 0; first < cnt; first += raw.size() / 4) {
      const size_t m = std::min(raw.size() / 4, cnt - first);
      if (std::fread(raw.data(), 1, m * 4, f.get()) != m * 4) {
        err = "netCDF read: " + path + " is truncated";
        return false;
      }
      for (size_t i = 0; i < m; ++i) {
        const uint32_t u = ((uint32_t)raw[4 * i] << 24) | ((uint32_t)raw[4 * i + 1] << 16) |
                           ((uint32_t)raw[4 * i + 2] << 8) | raw[4 * i + 3];
        std::memcpy(&values[first + i], &u, 4);
      }
    }
    shape = sh;
    return true;
  }
  err = r.ok ? "netCDF read: no variable " + name + " in " + path : "netCDF read: bad header in " + path;
  return false;
}

}  // namespace nc
}  // namespace umwm
