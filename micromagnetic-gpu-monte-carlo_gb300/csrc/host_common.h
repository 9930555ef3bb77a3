// host_common.h -- error reporting shared by the host-side translation units.
#pragma once
#include <string>
#include "../../include/mmc.h"

namespace mmc {

// Records `msg` as the calling thread's last error and returns `status`.
int fail(int status, const std::string& msg);
void clear_error();

// OVF helpers shared by the C ABI, the anneal loop and the tensor cache.
int ovf_read(const std::string& path, int nx, int ny, int nz, double dx, double dy, double dz,
             double* mx, double* my, double* mz);
int ovf_write(const std::string& path, int nx, int ny, int nz, double dx, double dy, double dz,
              const double* mx, const double* my, const double* mz, int format,
              const std::string& title, const std::string& labels = "m_x m_y m_z",
              const std::string& units = "1 1 1");

int config_load_ini(const std::string& path, mmc_config* cfg);
int config_validate(const mmc_config* cfg);
std::string config_format(const mmc_config* cfg);
void config_defaults(mmc_config* cfg);

}  // namespace mmc
