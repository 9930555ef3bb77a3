// ovf.cpp -- OOMMF vector field file reader and writer.
//
// Replaces parseOvfFile / writetoOvfFile (reference src/ovf_io.h:88-105, empty
// bodies in the published source).  The header handling follows the
// reference's parseHeaderLine (src/ovf_io.h:66-85: "# key: value", key and
// value lower-cased, value cut at a second '#') and its OvfInfo equality test
// (src/ovf_io.h:35-64: equal node counts, step sizes equal within 1e-5
// relative).  The data layout is the OVF one (src/ovf_io.h:156-164): value
// triples, x index fastest, then y, then z.
//
// Formats read: OVF 2.0 ("Data Text", "Data Binary 4", "Data Binary 8",
// little-endian) and OVF 1.0 rectangular meshes (binary data big-endian; the
// stored values times "valuemultiplier" are the field).  Header keys other
// than the node counts, step sizes, valuedim, meshtype and valuemultiplier
// (Title, Desc, units, extents, boundary, "##" comments) are skipped.
// Format written: OVF 2.0, binary 4 / binary 8 / text.
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "host_common.h"

namespace mmc {

namespace {

std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}
std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

// "# key: value # comment" -> (key, value), both lower-cased and trimmed.
bool header_kv(const std::string& line, std::string* key, std::string* val) {
  size_t c = line.find(':');
  if (c == std::string::npos) return false;
  std::string k = line.substr(0, c);
  std::string v = line.substr(c + 1);
  size_t h = v.find('#');
  if (h != std::string::npos) v = v.substr(0, h);
  size_t p = 0;
  while (p < k.size() && (k[p] == '#' || std::isspace((unsigned char)k[p]))) ++p;
  *key = lower(trim(k.substr(p)));
  *val = lower(trim(v));
  return true;
}

bool step_close(double a, double b) { return std::fabs(a - b) <= 1e-5 * (std::fabs(a) + std::fabs(b)); }

uint32_t load_u32(const unsigned char* p, bool big) {
  return big ? ((uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | (uint32_t)p[3])
             : ((uint32_t)p[3] << 24 | (uint32_t)p[2] << 16 | (uint32_t)p[1] << 8 | (uint32_t)p[0]);
}
uint64_t load_u64(const unsigned char* p, bool big) {
  uint64_t a = load_u32(p, big), b = load_u32(p + 4, big);
  return big ? (a << 32 | b) : (b << 32 | a);
}
float as_f32(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
double as_f64(uint64_t u) {
  double d;
  std::memcpy(&d, &u, 8);
  return d;
}
void store_u32_le(unsigned char* p, uint32_t u) {
  p[0] = (unsigned char)u;
  p[1] = (unsigned char)(u >> 8);
  p[2] = (unsigned char)(u >> 16);
  p[3] = (unsigned char)(u >> 24);
}

}  // namespace

int ovf_read(const std::string& path, int nx, int ny, int nz, double dx, double dy, double dz,
             double* mx, double* my, double* mz) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return fail(MMC_ERR_IO, "cannot open OVF file: " + path);
  std::string buf((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  size_t pos = 0;
  auto next_line = [&](std::string* out) -> bool {
    if (pos >= buf.size()) return false;
    size_t e = buf.find('\n', pos);
    if (e == std::string::npos) e = buf.size();
    *out = buf.substr(pos, e - pos);
    if (!out->empty() && out->back() == '\r') out->pop_back();
    pos = e + 1;
    return true;
  };
  std::string line;
  if (!next_line(&line)) return fail(MMC_ERR_IO, path + ": empty file");
  std::string first = lower(line);
  int version = 0;
  if (first.find("oommf ovf 2.0") != std::string::npos) version = 2;
  else if (first.find("oommf") != std::string::npos &&
           first.find("rectangular mesh v1.0") != std::string::npos) version = 1;
  else if (first.find("oommf") != std::string::npos && first.find("mesh v1") != std::string::npos)
    version = 1;
  if (!version) return fail(MMC_ERR_IO, path + ": not an OVF 1.0/2.0 file");

  long long xn = -1, yn = -1, zn = -1;
  double xs = -1, ys = -1, zs = -1;
  int valuedim = 3;
  double multiplier = 1.0;  // OVF 1.0: stored values times valuemultiplier are the field
  std::string meshtype = "rectangular";
  std::string data_kind;
  while (next_line(&line)) {
    std::string t = trim(line);
    if (t.empty()) continue;
    if (t[0] != '#') return fail(MMC_ERR_IO, path + ": unexpected line before data: " + t);
    std::string k, v;
    if (!header_kv(t, &k, &v)) continue;
    if (k == "xnodes") xn = std::atoll(v.c_str());
    else if (k == "ynodes") yn = std::atoll(v.c_str());
    else if (k == "znodes") zn = std::atoll(v.c_str());
    else if (k == "xstepsize") xs = std::atof(v.c_str());
    else if (k == "ystepsize") ys = std::atof(v.c_str());
    else if (k == "zstepsize") zs = std::atof(v.c_str());
    else if (k == "valuedim") valuedim = std::atoi(v.c_str());
    else if (k == "valuemultiplier" && version == 1) multiplier = std::atof(v.c_str());
    else if (k == "meshtype") meshtype = v;
    else if (k == "begin" && v.rfind("data", 0) == 0) {
      data_kind = v;
      break;
    }
  }
  if (data_kind.empty()) return fail(MMC_ERR_IO, path + ": no data segment");
  if (meshtype != "rectangular") return fail(MMC_ERR_IO, path + ": only rectangular meshes are supported");
  if (valuedim != 3) return fail(MMC_ERR_IO, path + ": valuedim must be 3");
  if (xn != nx || yn != ny || zn != nz || !step_close(xs, dx) || !step_close(ys, dy) ||
      !step_close(zs, dz)) {
    char msg[512];
    std::snprintf(msg, sizeof msg,
                  "%s: mesh %lldx%lldx%lld step %g %g %g does not match %dx%dx%d step %g %g %g",
                  path.c_str(), xn, yn, zn, xs, ys, zs, nx, ny, nz, dx, dy, dz);
    return fail(MMC_ERR_IO, msg);
  }
  const size_t n = (size_t)nx * ny * nz;
  if (data_kind.find("text") != std::string::npos) {
    size_t got = 0;
    std::vector<double> vals(3 * n);
    while (got < 3 * n && next_line(&line)) {
      std::string t = trim(line);
      if (t.empty() || t[0] == '#') continue;
      const char* s = t.c_str();
      while (*s && got < 3 * n) {
        char* e = nullptr;
        double d = std::strtod(s, &e);
        if (e == s) return fail(MMC_ERR_IO, path + ": bad number in text data");
        vals[got++] = d;
        s = e;
        while (*s && std::isspace((unsigned char)*s)) ++s;
      }
    }
    if (got != 3 * n) return fail(MMC_ERR_IO, path + ": truncated text data");
    for (size_t i = 0; i < n; ++i) {
      mx[i] = multiplier * vals[3 * i];
      my[i] = multiplier * vals[3 * i + 1];
      mz[i] = multiplier * vals[3 * i + 2];
    }
    return MMC_OK;
  }
  int width = 0;
  if (data_kind.find("binary 4") != std::string::npos || data_kind.find("binary4") != std::string::npos)
    width = 4;
  else if (data_kind.find("binary 8") != std::string::npos || data_kind.find("binary8") != std::string::npos)
    width = 8;
  else
    return fail(MMC_ERR_IO, path + ": unsupported data kind '" + data_kind + "'");
  const size_t need = (size_t)width * (1 + 3 * n);
  if (buf.size() < pos || buf.size() - pos < need) return fail(MMC_ERR_IO, path + ": truncated binary data");
  const unsigned char* p = reinterpret_cast<const unsigned char*>(buf.data()) + pos;
  bool big = false;
  if (width == 4) {
    if (as_f32(load_u32(p, false)) == 1234567.0f) big = false;
    else if (as_f32(load_u32(p, true)) == 1234567.0f) big = true;
    else return fail(MMC_ERR_IO, path + ": bad binary-4 check value");
  } else {
    if (as_f64(load_u64(p, false)) == 123456789012345.0) big = false;
    else if (as_f64(load_u64(p, true)) == 123456789012345.0) big = true;
    else return fail(MMC_ERR_IO, path + ": bad binary-8 check value");
  }
  p += width;
  for (size_t i = 0; i < n; ++i) {
    double v[3];
    for (int c = 0; c < 3; ++c) {
      const unsigned char* q = p + (3 * i + c) * (size_t)width;
      v[c] = width == 4 ? (double)as_f32(load_u32(q, big)) : as_f64(load_u64(q, big));
    }
    mx[i] = multiplier * v[0];
    my[i] = multiplier * v[1];
    mz[i] = multiplier * v[2];
  }
  return MMC_OK;
}

int ovf_write(const std::string& path, int nx, int ny, int nz, double dx, double dy, double dz,
              const double* mx, const double* my, const double* mz, int format,
              const std::string& title, const std::string& labels, const std::string& units) {
  if (format < 0 || format > 2) return fail(MMC_ERR_INVALID, "bad OVF format");
  std::ofstream out(path, std::ios::binary | std::ios::trunc);
  if (!out) return fail(MMC_ERR_IO, "cannot write OVF file: " + path);
  const char* kind = format == MMC_OVF_BINARY4 ? "Binary 4" : format == MMC_OVF_BINARY8 ? "Binary 8" : "Text";
  std::ostringstream h;
  h.precision(17);
  h << "# OOMMF OVF 2.0\n# Segment count: 1\n# Begin: Segment\n# Begin: Header\n";
  h << "# Title: " << (title.empty() ? std::string("m") : title) << "\n";
  h << "# meshtype: rectangular\n# meshunit: m\n";
  h << "# xmin: 0\n# ymin: 0\n# zmin: 0\n";
  h << "# xmax: " << nx * dx << "\n# ymax: " << ny * dy << "\n# zmax: " << nz * dz << "\n";
  h << "# valuedim: 3\n# valuelabels: " << labels << "\n# valueunits: " << units << "\n";
  h << "# xbase: " << 0.5 * dx << "\n# ybase: " << 0.5 * dy << "\n# zbase: " << 0.5 * dz << "\n";
  h << "# xnodes: " << nx << "\n# ynodes: " << ny << "\n# znodes: " << nz << "\n";
  h << "# xstepsize: " << dx << "\n# ystepsize: " << dy << "\n# zstepsize: " << dz << "\n";
  h << "# End: Header\n# Begin: Data " << kind << "\n";
  std::string hs = h.str();
  out.write(hs.data(), (std::streamsize)hs.size());
  const size_t n = (size_t)nx * ny * nz;
  if (format == MMC_OVF_TEXT) {
    char line[128];
    for (size_t i = 0; i < n; ++i) {
      int len = std::snprintf(line, sizeof line, "%.17g %.17g %.17g\n", mx[i], my[i], mz[i]);
      out.write(line, len);
    }
  } else if (format == MMC_OVF_BINARY4) {
    std::vector<unsigned char> b(4 * (1 + 3 * n));
    float chk = 1234567.0f;
    uint32_t u;
    std::memcpy(&u, &chk, 4);
    store_u32_le(b.data(), u);
    for (size_t i = 0; i < n; ++i) {
      const double v[3] = {mx[i], my[i], mz[i]};
      for (int c = 0; c < 3; ++c) {
        float f = (float)v[c];
        std::memcpy(&u, &f, 4);
        store_u32_le(b.data() + 4 * (1 + 3 * i + c), u);
      }
    }
    out.write(reinterpret_cast<const char*>(b.data()), (std::streamsize)b.size());
  } else {
    std::vector<unsigned char> b(8 * (1 + 3 * n));
    auto put = [&](size_t slot, double d) {
      uint64_t u;
      std::memcpy(&u, &d, 8);
      store_u32_le(b.data() + 8 * slot, (uint32_t)u);
      store_u32_le(b.data() + 8 * slot + 4, (uint32_t)(u >> 32));
    };
    put(0, 123456789012345.0);
    for (size_t i = 0; i < n; ++i) {
      put(1 + 3 * i, mx[i]);
      put(2 + 3 * i, my[i]);
      put(3 + 3 * i, mz[i]);
    }
    out.write(reinterpret_cast<const char*>(b.data()), (std::streamsize)b.size());
  }
  std::string tail = std::string("\n# End: Data ") + kind + "\n# End: Segment\n";
  if (format == MMC_OVF_TEXT) tail = std::string("# End: Data ") + kind + "\n# End: Segment\n";
  out.write(tail.data(), (std::streamsize)tail.size());
  if (!out) return fail(MMC_ERR_IO, "write failed: " + path);
  return MMC_OK;
}

}  // namespace mmc
