// ini.cpp -- configuration file reader and echo.
//
// Replaces parse_input_ini (reference src/parse_input_ini.h:15-47, whose body
// is empty in the published source; it was written against
// boost::property_tree's ini reader) and cout_input_ini (:49-114).  The key
// set, names and value types are the reference's (:15-41, README.md:44-86):
// `key = value` lines, ';' or '#' full-line comments, [section] headers
// ignored.  The optional keys added by this library are listed in
// include/mmc.h and default to the reference's behaviour.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <string>

#include "host_common.h"

namespace mmc {

namespace {

thread_local std::string g_last_error;

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

bool parse_ll(const std::string& v, long long* out) {
  if (v.empty()) return false;
  errno = 0;
  char* end = nullptr;
  long long x = std::strtoll(v.c_str(), &end, 10);
  if (errno != 0 || end == v.c_str() || *end != '\0') {
    // accept integral values written in floating-point form, e.g. "1e4"
    char* e2 = nullptr;
    double d = std::strtod(v.c_str(), &e2);
    if (e2 == v.c_str() || *e2 != '\0' || !std::isfinite(d) || d != std::floor(d) ||
        std::fabs(d) > 9.0e18)
      return false;
    x = (long long)d;
  }
  *out = x;
  return true;
}

bool parse_double(const std::string& v, double* out) {
  if (v.empty()) return false;
  char* end = nullptr;
  double x = std::strtod(v.c_str(), &end);
  if (end == v.c_str() || *end != '\0' || !std::isfinite(x)) return false;
  *out = x;
  return true;
}

bool parse_bool(const std::string& v0, int* out) {
  std::string v = lower(v0);
  if (v == "true" || v == "1" || v == "yes" || v == "on") {
    *out = 1;
    return true;
  }
  if (v == "false" || v == "0" || v == "no" || v == "off") {
    *out = 0;
    return true;
  }
  return false;
}

enum Kind { K_INT, K_LL, K_DOUBLE, K_BOOL, K_STR };
struct KeyDef {
  const char* name;
  Kind kind;
  size_t offset;
  bool required;
};

#define KD(field, kind, req) {#field, kind, offsetof(mmc_config, field), req}
const KeyDef kKeys[] = {
    KD(nx, K_INT, true), KD(ny, K_INT, true), KD(nz, K_INT, true),
    KD(dx, K_DOUBLE, true), KD(dy, K_DOUBLE, true), KD(dz, K_DOUBLE, true),
    KD(Bextx, K_DOUBLE, true), KD(Bexty, K_DOUBLE, true), KD(Bextz, K_DOUBLE, true),
    KD(pbc_x, K_INT, true), KD(pbc_y, K_INT, true), KD(pbc_z, K_INT, true),
    KD(ms, K_DOUBLE, true), KD(Aex, K_DOUBLE, true), KD(Dind, K_DOUBLE, true),
    KD(anisUx, K_DOUBLE, true), KD(anisUy, K_DOUBLE, true), KD(anisUz, K_DOUBLE, true),
    KD(Ku1, K_DOUBLE, true),
    KD(use_random_init, K_BOOL, true), KD(randomseed, K_LL, true), KD(ovf_filename, K_STR, true),
    KD(Temperature_start, K_DOUBLE, true), KD(Temperature_end, K_DOUBLE, true),
    KD(Temperature_step, K_DOUBLE, true), KD(Temperature_use_exp, K_BOOL, true),
    KD(circle_per_stage, K_LL, true), KD(terminal_output_period, K_LL, true),
    KD(energy_output_period, K_LL, true), KD(ms_output_period, K_LL, true),
    KD(rand_block_size, K_INT, true), KD(cal_demag_flag, K_BOOL, true),
    // optional keys of this library
    KD(use_reference_pi, K_BOOL, false), KD(tensor_cache, K_STR, false), KD(fused_band, K_INT, false),
    KD(tensor_far_radius, K_INT, false), KD(debug_h_field, K_BOOL, false), KD(tensor_sum, K_INT, false),
};
#undef KD

}  // namespace

int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}
void clear_error() { g_last_error.clear(); }
const char* last_error_cstr() { return g_last_error.c_str(); }

void config_defaults(mmc_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->nx = 256; c->ny = 256; c->nz = 1;
  c->dx = 1e-9; c->dy = 1e-9; c->dz = 0.8e-9;
  c->Bextx = 0; c->Bexty = 0; c->Bextz = 0.3;
  c->pbc_x = 20; c->pbc_y = 20; c->pbc_z = 0;
  c->ms = 1.6e6; c->Aex = 16e-12; c->Dind = 6e-3;
  c->anisUx = 0; c->anisUy = 0; c->anisUz = 1; c->Ku1 = 2e6;
  c->use_random_init = 1;
  c->randomseed = 256;
  c->Temperature_start = 1400; c->Temperature_end = 40; c->Temperature_step = 0.90;
  c->Temperature_use_exp = 1;
  c->circle_per_stage = 100000;
  c->terminal_output_period = 10001;
  c->energy_output_period = 10001;
  c->ms_output_period = 10001;
  c->rand_block_size = 40;
  c->cal_demag_flag = 1;
  c->precision = 32;
  c->ovf_format = MMC_OVF_BINARY4;
  c->use_reference_pi = 0;
  c->tensor_sum = 1;
}

int config_validate(const mmc_config* c) {
  if (c->nx < 1 || c->ny < 1 || c->nz < 1)
    return fail(MMC_ERR_CONFIG, "nx, ny, nz must be >= 1");
  if ((long long)c->nx * c->ny * c->nz >= (1LL << 31))
    return fail(MMC_ERR_CONFIG, "lattice of 2^31 cells or more");
  if (!(c->dx > 0) || !(c->dy > 0) || !(c->dz > 0))
    return fail(MMC_ERR_CONFIG, "dx, dy, dz must be > 0");
  if (!(c->ms > 0)) return fail(MMC_ERR_CONFIG, "ms must be > 0");
  if (c->precision != 32 && c->precision != 64)
    return fail(MMC_ERR_CONFIG, "precision must be 32 or 64");
  if (c->ovf_format < 0 || c->ovf_format > 2) return fail(MMC_ERR_CONFIG, "bad ovf_format");
  if (c->sweep_engine < 0 || c->sweep_engine > 2) return fail(MMC_ERR_CONFIG, "bad sweep_engine");
  if (c->fused_band < 0 || c->fused_band > 60) return fail(MMC_ERR_CONFIG, "fused_band must be in [0, 60]");
  if (c->tensor_far_radius != 0 && (c->tensor_far_radius < 12 || c->tensor_far_radius > 1000000))
    return fail(MMC_ERR_CONFIG, "tensor_far_radius must be 0 (off) or in [12, 1e6] cells");
  if (c->tensor_sum != 0 && c->tensor_sum != 1) return fail(MMC_ERR_CONFIG, "tensor_sum must be 0 or 1");
  if (c->circle_per_stage < 0) return fail(MMC_ERR_CONFIG, "circle_per_stage must be >= 0");
  if (c->terminal_output_period < 1 || c->energy_output_period < 1 || c->ms_output_period < 1)
    return fail(MMC_ERR_CONFIG, "output periods must be >= 1");
  if (c->Temperature_use_exp) {
    if (!(c->Temperature_step > 0 && c->Temperature_step < 1) && c->Temperature_start > c->Temperature_end)
      return fail(MMC_ERR_CONFIG,
                  "Temperature_use_exp requires 0 < Temperature_step < 1 (the loop would not end)");
  } else {
    if (!(c->Temperature_step > 0) && c->Temperature_start > c->Temperature_end)
      return fail(MMC_ERR_CONFIG, "Temperature_step must be > 0 (the loop would not end)");
  }
  if (!std::isfinite(c->Temperature_start) || !std::isfinite(c->Temperature_end))
    return fail(MMC_ERR_CONFIG, "temperatures must be finite");
  return MMC_OK;
}

int config_load_ini(const std::string& path, mmc_config* cfg) {
  std::ifstream in(path);
  if (!in) return fail(MMC_ERR_IO, "cannot open ini file: " + path);
  mmc_config c;
  config_defaults(&c);
  std::set<std::string> seen;
  std::string line;
  int lineno = 0;
  while (std::getline(in, line)) {
    ++lineno;
    std::string t = trim(line);
    if (t.empty() || t[0] == ';' || t[0] == '#') continue;
    if (t[0] == '[') continue;  // section header
    size_t eq = t.find('=');
    if (eq == std::string::npos)
      return fail(MMC_ERR_CONFIG, path + ":" + std::to_string(lineno) + ": expected key = value");
    std::string key = trim(t.substr(0, eq));
    std::string val = trim(t.substr(eq + 1));
    if (seen.count(key))
      return fail(MMC_ERR_CONFIG, path + ":" + std::to_string(lineno) + ": duplicate key " + key);
    seen.insert(key);
    char* base = reinterpret_cast<char*>(&c);
    // optional keys with enumerated values
    if (key == "precision") {
      std::string v = lower(val);
      if (v == "32" || v == "fp32" || v == "float" || v == "single") c.precision = 32;
      else if (v == "64" || v == "fp64" || v == "double") c.precision = 64;
      else return fail(MMC_ERR_CONFIG, "precision must be fp32 or fp64, got " + val);
      continue;
    }
    if (key == "ovf_format") {
      std::string v = lower(val);
      if (v == "binary4" || v == "binary 4") c.ovf_format = MMC_OVF_BINARY4;
      else if (v == "binary8" || v == "binary 8") c.ovf_format = MMC_OVF_BINARY8;
      else if (v == "text") c.ovf_format = MMC_OVF_TEXT;
      else return fail(MMC_ERR_CONFIG, "ovf_format must be binary4, binary8 or text, got " + val);
      continue;
    }
    if (key == "sweep_engine") {
      std::string v = lower(val);
      if (v == "auto") c.sweep_engine = MMC_ENGINE_AUTO;
      else if (v == "kernels") c.sweep_engine = MMC_ENGINE_KERNELS;
      else if (v == "fused") c.sweep_engine = MMC_ENGINE_FUSED;
      else return fail(MMC_ERR_CONFIG, "sweep_engine must be auto, kernels or fused, got " + val);
      continue;
    }
    const KeyDef* kd = nullptr;
    for (const auto& k : kKeys)
      if (key == k.name) kd = &k;
    if (!kd) return fail(MMC_ERR_CONFIG, path + ":" + std::to_string(lineno) + ": unknown key " + key);
    bool ok = true;
    switch (kd->kind) {
      case K_INT: {
        long long v;
        ok = parse_ll(val, &v) && v >= INT32_MIN && v <= INT32_MAX;
        if (ok) *reinterpret_cast<int*>(base + kd->offset) = (int)v;
        break;
      }
      case K_LL: {
        long long v;
        ok = parse_ll(val, &v);
        if (ok) *reinterpret_cast<long long*>(base + kd->offset) = v;
        break;
      }
      case K_DOUBLE: {
        double v;
        ok = parse_double(val, &v);
        if (ok) *reinterpret_cast<double*>(base + kd->offset) = v;
        break;
      }
      case K_BOOL: {
        int v;
        ok = parse_bool(val, &v);
        if (ok) *reinterpret_cast<int*>(base + kd->offset) = v;
        break;
      }
      case K_STR: {
        if (val.size() >= 1024) ok = false;
        else {
          char* dst = base + kd->offset;
          std::memset(dst, 0, 1024);
          std::memcpy(dst, val.data(), val.size());
        }
        break;
      }
    }
    if (!ok)
      return fail(MMC_ERR_CONFIG,
                  path + ":" + std::to_string(lineno) + ": bad value for " + key + ": " + val);
  }
  std::string missing;
  for (const auto& k : kKeys)
    if (k.required && !seen.count(k.name)) missing += std::string(missing.empty() ? "" : ", ") + k.name;
  if (!missing.empty()) return fail(MMC_ERR_CONFIG, path + ": missing keys: " + missing);
  int st = config_validate(&c);
  if (st != MMC_OK) return st;
  *cfg = c;
  return MMC_OK;
}

std::string config_format(const mmc_config* c) {
  std::ostringstream o;
  o << "====================display ini file============\n";
  o << "nx: " << c->nx << "\nny: " << c->ny << "\nnz: " << c->nz << "\n";
  o << "dx: " << c->dx << "\ndy: " << c->dy << "\ndz: " << c->dz << "\n";
  o << "Bextx: " << c->Bextx << "\nBexty: " << c->Bexty << "\nBextz: " << c->Bextz << "\n";
  o << "pbc_x: " << c->pbc_x << "\npbc_y: " << c->pbc_y << "\npbc_z: " << c->pbc_z << "\n";
  o << "ms: " << c->ms << "\nAex: " << c->Aex << "\nDind: " << c->Dind << "\n";
  o << "anisUx: " << c->anisUx << "\nanisUy: " << c->anisUy << "\nanisUz: " << c->anisUz << "\n";
  o << "Ku1: " << c->Ku1 << "\n";
  o << "use_random_init: " << c->use_random_init << "\nrandomseed: " << c->randomseed << "\n";
  o << "ovf_filename: " << c->ovf_filename << "\n";
  o << "Temperature_start: " << c->Temperature_start << "\nTemperature_end: " << c->Temperature_end
    << "\nTemperature_step: " << c->Temperature_step
    << "\nTemperature_use_exp: " << c->Temperature_use_exp << "\n";
  o << "circle_per_stage: " << c->circle_per_stage
    << "\nterminal_output_period: " << c->terminal_output_period
    << "\nenergy_output_period: " << c->energy_output_period
    << "\nms_output_period: " << c->ms_output_period << "\n";
  o << "rand_block_size: " << c->rand_block_size << "\ncal_demag_flag: " << c->cal_demag_flag << "\n";
  o << "precision: fp" << c->precision << "\n";
  o << "---------------------END display ini file------------\n";
  return o.str();
}

}  // namespace mmc
