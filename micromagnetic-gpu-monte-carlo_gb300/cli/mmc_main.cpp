// mmc_main.cpp -- command-line driver, a drop-in for the reference binary.
//
//   mmc <cfg.ini> [-gpu=N] [-tensorcache="/path/"] [-farm-Bz=b1,b2,...] [-farm-D=d1,d2,...]
//       [-farm-seeds=N]
//
// Argument handling follows src/main.cu:97-105 and src/GPU_selector.h:11-76:
// the first argument not starting with '-' is the ini file, -gpu=N picks the
// device (default 0), -tensorcache= names the demag-tensor cache folder.
// Outputs go to <ini dir>/<ini stem>.output/ (src/main.cu:193-231): energy.txt
// and the OVF snapshots.  Ctrl-C stops the anneal at the next sweep boundary.
//
// -farm-Bz= / -farm-D= / -farm-seeds= (not in the reference) anneal a parameter
// sweep or a seed ensemble from the same ini: N replicas (-farm-seeds, default
// 1) per (B_z, D) pair, replica k seeded randomseed + k, all in one batch on
// the GPU; replica k writes into replica_<kkk>/ of the output folder and
// farm.txt lists k, B_z, D and the seed.
#include <algorithm>
#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <unistd.h>
#include <climits>

#include "mmc.h"

static mmc_handle* g_handle = nullptr;
static mmc_batch* g_batch = nullptr;

static void on_sigint(int) {
  if (g_handle) mmc_request_stop(g_handle);
  if (g_batch) mmc_batch_request_stop(g_batch);
}

// "a,b,c" -> values; false on a malformed number
static bool parse_list(const std::string& s, std::vector<double>& out) {
  size_t i = 0;
  while (i <= s.size()) {
    size_t j = s.find(',', i);
    if (j == std::string::npos) j = s.size();
    const std::string tok = s.substr(i, j - i);
    char* end = nullptr;
    const double v = std::strtod(tok.c_str(), &end);
    if (tok.empty() || *end != '\0') return false;
    out.push_back(v);
    i = j + 1;
  }
  return !out.empty();
}

// The parameter sweep: one batch of replicas, the stage loop for all of them.
static int run_farm(const mmc_config& cfg, int gpu, const std::vector<double>& bz, const std::vector<double>& dm,
                    int seeds, const std::string& out) {
  std::vector<mmc_config> cfgs;
  for (double b : bz)
    for (double d : dm)
      for (int s = 0; s < seeds; ++s) {
        mmc_config c = cfg;
        c.Bextz = b;
        c.Dind = d;
        if (cfg.randomseed >= 0) c.randomseed = cfg.randomseed + (long long)cfgs.size();
        cfgs.push_back(c);
      }
  std::printf("farm: %zu replicas\n", cfgs.size());
  int st = mmc_batch_create(cfgs.data(), (int)cfgs.size(), gpu, &g_batch);
  if (st != MMC_OK) return st;
  std::signal(SIGINT, on_sigint);
  if (cfg.cal_demag_flag) {
    std::printf("Calculating demag tensor...\n");
    st = mmc_batch_build_demag(g_batch, cfg.tensor_cache);
  }
  if (st == MMC_OK) st = mmc_batch_autotune(g_batch, 8, nullptr, nullptr);
  if (st == MMC_OK) {
    std::printf("Start...\n");
    st = mmc_batch_run_anneal(g_batch, out.c_str(), 1);
  }
  if (st == MMC_OK || st == MMC_ERR_INTERRUPTED) {
    FILE* fp = std::fopen((out + "/farm.txt").c_str(), "w");
    if (fp) {
      for (size_t k = 0; k < cfgs.size(); ++k)
        std::fprintf(fp, "%zu %g %g %lld\n", k, cfgs[k].Bextz, cfgs[k].Dind, cfgs[k].randomseed);
      std::fclose(fp);
    }
  }
  return st;
}

static std::string abspath(const std::string& p) {
  if (!p.empty() && p[0] == '/') return p;
  char buf[PATH_MAX];
  if (!getcwd(buf, sizeof buf)) return p;
  return std::string(buf) + "/" + p;
}

int main(int argc, char** argv) {
  setbuf(stdout, nullptr);
  if (argc == 1) {
    std::printf("need input file. \n");
    std::printf("arg format:  input_cfg_file.ini  -gpu=0   -tensorcache=\"/mnt/cachepath/\" \n");
    return 0;
  }
  std::string cfg_path, cache;
  int gpu = 0;
  std::vector<double> farm_bz, farm_d;
  int farm_seeds = 0;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (a.empty()) continue;
    if (a[0] != '-') {
      if (cfg_path.empty()) cfg_path = a;
      continue;
    }
    std::string key = a.substr(a.find_first_not_of('-'));
    if (key.rfind("gpu=", 0) == 0) {
      gpu = std::atoi(key.c_str() + 4);
      if (gpu < 0) {
        std::printf("Invalid command line parameter: -gpu=\n ");
        return 1;
      }
    } else if (key.rfind("tensorcache=", 0) == 0) {
      cache = key.substr(12);
      if (cache.size() >= 2 && cache.front() == '"' && cache.back() == '"') cache = cache.substr(1, cache.size() - 2);
    } else if (key.rfind("farm-Bz=", 0) == 0) {
      if (!parse_list(key.substr(8), farm_bz)) {
        std::printf("Invalid command line parameter: -farm-Bz=\n");
        return 1;
      }
    } else if (key.rfind("farm-D=", 0) == 0) {
      if (!parse_list(key.substr(7), farm_d)) {
        std::printf("Invalid command line parameter: -farm-D=\n");
        return 1;
      }
    } else if (key.rfind("farm-seeds=", 0) == 0) {
      char* end = nullptr;
      const long v = std::strtol(key.c_str() + 11, &end, 10);
      if (key.size() == 11 || *end != '\0' || v < 1 || v > 65535) {
        std::printf("Invalid command line parameter: -farm-seeds=\n");
        return 1;
      }
      farm_seeds = (int)v;
    }
  }
  cfg_path = abspath(cfg_path);
  std::printf("input_cfg_path is : %s\n", cfg_path.c_str());
  mmc_config cfg;
  int st = mmc_config_load_ini(cfg_path.c_str(), &cfg);
  if (st != MMC_OK) {
    std::fprintf(stderr, "error: %s\n", mmc_last_error());
    return 2;
  }
  if (!cache.empty()) {
    std::snprintf(cfg.tensor_cache, sizeof cfg.tensor_cache, "%s", cache.c_str());
    std::printf("cache path: %s\n", cache.c_str());
  }
  std::vector<char> echo(8192);
  mmc_config_format(&cfg, echo.data(), echo.size());
  std::fputs(echo.data(), stdout);

  std::string dir = cfg_path.substr(0, cfg_path.find_last_of('/'));
  std::string base = cfg_path.substr(cfg_path.find_last_of('/') + 1);
  std::string stem = base.substr(0, base.find_last_of('.'));
  std::string out = dir + "/" + stem + ".output";
  std::printf("output_path: %s\n", out.c_str());

  if (!farm_bz.empty() || !farm_d.empty() || farm_seeds > 0) {
    if (farm_bz.empty()) farm_bz.push_back(cfg.Bextz);
    if (farm_d.empty()) farm_d.push_back(cfg.Dind);
    if ((long long)farm_bz.size() * (long long)farm_d.size() * std::max(farm_seeds, 1) > 65535) {
      std::printf("Invalid command line parameters: more than 65535 farm replicas\n");
      return 1;
    }
    st = run_farm(cfg, gpu, farm_bz, farm_d, std::max(farm_seeds, 1), out);
    int rc = 0;
    if (st == MMC_ERR_INTERRUPTED) {
      std::printf("interrupted\n");
    } else if (st != MMC_OK) {
      std::fprintf(stderr, "error: %s\n", mmc_last_error());
      rc = 5;
    }
    mmc_batch_destroy(g_batch);
    g_batch = nullptr;
    return rc;
  }

  st = mmc_create(&cfg, gpu, &g_handle);
  if (st != MMC_OK) {
    std::fprintf(stderr, "error: %s\n", mmc_last_error());
    return 3;
  }
  int dims[3];
  mmc_padded_dims(&cfg, dims);
  std::printf("\nDimension: nx ny nz meshsize\n%d %d %d %lld\n", cfg.nx, cfg.ny, cfg.nz,
              (long long)cfg.nx * cfg.ny * cfg.nz);
  std::printf("nx_padded ny_padded nz_padded meshsize_padded\n%d %d %d %lld\n", dims[0], dims[1], dims[2],
              (long long)dims[0] * dims[1] * dims[2]);
  std::signal(SIGINT, on_sigint);
  if (cfg.cal_demag_flag) {
    std::printf("Calculating demag tensor...\n");
    st = mmc_build_demag(g_handle, cfg.tensor_cache);
    if (st != MMC_OK && st != MMC_ERR_INTERRUPTED) {
      std::fprintf(stderr, "error: %s\n", mmc_last_error());
      mmc_destroy(g_handle);
      return 4;
    }
    std::printf("Done.\n");
  }
  std::printf("Start...\n");
  if (st == MMC_OK) st = mmc_run_anneal(g_handle, out.c_str(), 1);
  int rc = 0;
  if (st == MMC_ERR_INTERRUPTED) {
    std::printf("interrupted\n");
  } else if (st != MMC_OK) {
    std::fprintf(stderr, "error: %s\n", mmc_last_error());
    rc = 5;
  }
  mmc_destroy(g_handle);
  g_handle = nullptr;
  return rc;
}
