// Visualisation output and checkpoints from device state (declared in
// include/mcell_gb300.h).
//
// Viz files follow VizOutputEvent (src4/viz_output_event.cpp:48-279): the name
// "<prefix>.<ascii|cellbin>.<iteration, zero-padded to the digits of the total>.dat";
// ASCII lines "name id x y z nx ny nz" (%.9g, um, zero normals for volume
// molecules); CellBlender binary: a uint version (1 or 2), then per species with
// molecules, in species order: the name length (uchar in version 1, uint in 2),
// the name, a uchar type (0 = volume), the count (version 1: 3 x molecules as a
// uint; version 2: molecules), version 2 only: the uint ids, then float x y z per
// molecule (um). Molecules are written in the engine's sorted order (the
// reference writes them in its own array order).
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <string>
#include <vector>

#include "mcg_batch.h"

namespace {

std::string iteration_string(uint64_t it, uint64_t total) {
  // VizOutputEvent::iterations_to_string
  uint64_t lli = 10;
  int ndigits = 1;
  for (; lli <= total && ndigits < 20; ndigits++) lli *= 10;
  char buf[32];
  std::snprintf(buf, sizeof(buf), "%0*llu", ndigits, (unsigned long long)it);
  return buf;
}

int write_viz(mcg::DeviceEngine* dev, uint32_t rep, const char* prefix, int mode, uint32_t nsp,
              const char* const* names, uint64_t iteration, uint64_t total, double lu, std::string& err) {
  if (mode != MCG_VIZ_ASCII && mode != MCG_VIZ_CELLBLENDER_V1 && mode != MCG_VIZ_CELLBLENDER_V2) {
    err = "unknown viz mode";
    return MCG_ERR_ARG;
  }
  uint64_t n = 0;
  int rc = dev->download(rep, 0, nullptr, nullptr, nullptr, &n, err);
  if (rc) return rc;
  std::vector<double> pos(3 * n);
  std::vector<uint32_t> sp(n);
  std::vector<uint64_t> ids(n);
  rc = dev->download(rep, n, pos.data(), sp.data(), ids.data(), &n, err);
  if (rc) return rc;
  const bool ascii = mode == MCG_VIZ_ASCII;
  const std::string path =
      std::string(prefix) + (ascii ? ".ascii." : ".cellbin.") + iteration_string(iteration, total) + ".dat";
  std::error_code ec;
  const std::filesystem::path parent = std::filesystem::path(path).parent_path();
  if (!parent.empty()) std::filesystem::create_directories(parent, ec);
  FILE* f = std::fopen(path.c_str(), ascii ? "w" : "wb");
  if (!f) {
    err = "cannot open " + path;
    return MCG_ERR_ARG;
  }
  bool ok = true;
  if (ascii) {
    for (uint64_t i = 0; i < n && ok; i++)
      ok = std::fprintf(f, "%s %u %.9g %.9g %.9g %.9g %.9g %.9g\n", names[sp[i]], (unsigned)ids[i], pos[3 * i] * lu,
                        pos[3 * i + 1] * lu, pos[3 * i + 2] * lu, 0.0, 0.0, 0.0) > 0;
  } else {
    const uint32_t ver = mode == MCG_VIZ_CELLBLENDER_V2 ? 2 : 1;
    ok = std::fwrite(&ver, sizeof(uint32_t), 1, f) == 1;
    for (uint32_t a = 0; a < nsp && ok; a++) {
      std::vector<uint64_t> idx;
      for (uint64_t i = 0; i < n; i++)
        if (sp[i] == a) idx.push_back(i);
      if (idx.empty()) continue;
      const size_t len = std::strlen(names[a]);
      if (ver == 1) {
        const unsigned char l8 = (unsigned char)len;
        ok = ok && std::fwrite(&l8, 1, 1, f) == 1;
      } else {
        const uint32_t l32 = (uint32_t)len;
        ok = ok && std::fwrite(&l32, sizeof(uint32_t), 1, f) == 1;
      }
      ok = ok && std::fwrite(names[a], 1, len, f) == len;
      const unsigned char type = 0;  // volume molecules
      ok = ok && std::fwrite(&type, 1, 1, f) == 1;
      const uint32_t count = ver == 1 ? (uint32_t)(3 * idx.size()) : (uint32_t)idx.size();
      ok = ok && std::fwrite(&count, sizeof(uint32_t), 1, f) == 1;
      if (ver == 2)
        for (uint64_t i : idx) {
          const uint32_t id = (uint32_t)ids[i];
          ok = ok && std::fwrite(&id, sizeof(uint32_t), 1, f) == 1;
        }
      for (uint64_t i : idx) {
        const float xyz[3] = {(float)(pos[3 * i] * lu), (float)(pos[3 * i + 1] * lu), (float)(pos[3 * i + 2] * lu)};
        ok = ok && std::fwrite(xyz, sizeof(float), 3, f) == 3;
      }
    }
  }
  if (std::fclose(f) != 0) ok = false;
  if (!ok) {
    err = "writing " + path + " failed";
    return MCG_ERR_ARG;
  }
  return MCG_OK;
}

}  // namespace

extern "C" {

int mcg_write_viz(mcg_engine* e, const char* prefix, int mode, const char* const* species_names, uint64_t iteration,
                  uint64_t total_iterations, double length_unit_um) {
  if (!e || !prefix || !species_names || !(length_unit_um > 0)) return MCG_ERR_ARG;
  if (!e->dev) {
    e->err = "mcg_write_viz needs a prepared engine";
    return MCG_ERR_ARG;
  }
  std::string err;
  int rc = write_viz(e->dev, 0, prefix, mode, e->cfg.n_species, species_names, iteration, total_iterations,
                     length_unit_um, err);
  if (rc) e->err = err;
  return rc;
}

int mcg_batch_write_viz(mcg_batch* b, uint32_t replica, const char* prefix, int mode, const char* const* species_names,
                        uint64_t iteration, uint64_t total_iterations, double length_unit_um) {
  if (!b || !prefix || !species_names || !(length_unit_um > 0)) return MCG_ERR_ARG;
  if (!b->dev) {
    b->err = "batch has no device engine";
    return MCG_ERR_CUDA;
  }
  std::string err;
  int rc = write_viz(b->dev, replica, prefix, mode, b->cfg.n_species, species_names, iteration, total_iterations,
                     length_unit_um, err);
  if (rc) b->err = err;
  return rc;
}

}  // extern "C"
