// mmc_main.cpp -- command-line driver, a drop-in for the reference binary.
//
//   mmc <cfg.ini> [-gpu=N] [-tensorcache="/path/"]
//
// Argument handling follows src/main.cu:97-105 and src/GPU_selector.h:11-76:
// the first argument not starting with '-' is the ini file, -gpu=N picks the
// device (default 0), -tensorcache= names the demag-tensor cache folder.
// Outputs go to <ini dir>/<ini stem>.output/ (src/main.cu:193-231): energy.txt
// and the OVF snapshots.  Ctrl-C stops the anneal at the next sweep boundary.
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

static void on_sigint(int) {
  if (g_handle) mmc_request_stop(g_handle);
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
