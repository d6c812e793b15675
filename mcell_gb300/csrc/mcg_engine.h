// Device engine interface shared by the fp64 and fp32 translation units and the C ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "mcg_setup.h"

namespace mcg {

struct ChemHost {
  uint32_t nsp = 0;
  double space_step[16] = {0};
  double unimol_k[16];
  int uni_prod[16][2];
  double bimol_p[16][16];
  int bimol_prod[16][16][2];
  ChemHost() {
    for (int a = 0; a < 16; a++) {
      unimol_k[a] = -1;
      uni_prod[a][0] = uni_prod[a][1] = -1;
      for (int b = 0; b < 16; b++) {
        bimol_p[a][b] = -1;
        bimol_prod[a][b][0] = bimol_prod[a][b][1] = -1;
      }
    }
  }
};

class DeviceEngine {
 public:
  virtual ~DeviceEngine() {}
  virtual int init(const HostSetup& hs, const ChemHost& chem, const std::vector<uint8_t>& wall_class, uint64_t seed,
                   uint64_t capacity, std::string& err) = 0;
  virtual int add_molecules(uint64_t n, const double* pos, const uint32_t* species, uint64_t uid0,
                            std::string& err) = 0;
  virtual int step(uint32_t n, std::string& err) = 0;
  virtual int sync(std::string& err) = 0;
  virtual int counts(uint64_t* out, std::string& err) = 0;
  virtual int trajectory(uint32_t n, uint64_t* out, std::string& err) = 0;
  virtual int download(uint64_t cap, double* pos, uint32_t* species, uint64_t* ids, uint64_t* n_out,
                       std::string& err) = 0;
  virtual int trace(uint32_t n, const uint64_t* ids, const double* disp, const uint32_t* draws, uint32_t ndraws,
                    const double* rrf, const double* tst, double* out, std::string& err) = 0;
  // trace() on the fixed scratch of mcg_trace_static.cu (no device allocation)
  virtual int trace_static(uint32_t n, const uint64_t* ids, const double* disp, const uint32_t* draws,
                           uint32_t ndraws, const double* rrf, const double* tst, double* out, std::string& err) = 0;
  virtual void stats(uint64_t* iterations, uint64_t* mol_steps, uint64_t* launches) = 0;
  virtual void set_options(int use_graphs, int profile) = 0;
  virtual int profile(double* out, std::string& err) = 0;
  virtual int debug_molecule(uint64_t uid, std::string& err) = 0;
  virtual int debug_log(double* out, std::string& err) = 0;
  virtual int escapes(double* out, uint32_t cap, uint32_t* n, std::string& err) = 0;
};

DeviceEngine* make_engine_f64();
DeviceEngine* make_engine_f32();

// maps device status bits to the ABI error codes (0 if clean)
int status_to_error(uint32_t status, std::string& err);

}  // namespace mcg
