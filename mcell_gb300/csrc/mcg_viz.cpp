// Visualisation and count output from device state (declared in
// include/mcell_gb300.h).
//
// Count files follow CountBuffer (src4/count_buffer.cpp:30-128): DAT lines
// "time value" with C++ stream defaults, GDAT a '#' header of right-aligned names
// and rows of scientific numbers with two-digit exponents.
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
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <sstream>
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

// CountBuffer's GDAT number (count_buffer.cpp:35-61): scientific with 8 decimals and
// a signed two-digit exponent
std::string gdat_number(double d) {
  std::stringstream ss;
  ss << std::scientific << std::setprecision(8) << d;
  const std::string s = ss.str();
  const size_t pos = s.find('e');
  int exponent = std::stoi(s.substr(pos + 1));
  std::ostringstream out;
  out << s.substr(0, pos) << "e" << (exponent >= 0 ? "+" : "-") << std::setfill('0') << std::setw(2)
      << (exponent >= 0 ? exponent : -exponent);
  return out.str();
}

int write_counts(mcg::DeviceEngine* dev, uint32_t rep, uint32_t nsp, const char* prefix, int format,
                 uint32_t n_it, uint32_t every, double dt, uint32_t ncol, const uint32_t* species,
                 const int32_t* objects, const char* const* names, std::string& err) {
  if (format != MCG_COUNTS_DAT && format != MCG_COUNTS_GDAT) {
    err = "unknown count format";
    return MCG_ERR_ARG;
  }
  if (every == 0 || ncol == 0 || !species || !objects || !names || !(dt > 0)) {
    err = "mcg_write_counts: every, columns, species, objects, names and time step are required";
    return MCG_ERR_ARG;
  }
  uint32_t n_cv = 0;
  uint64_t ran = 0;  // rows of the replica's trajectories so far
  int rc = dev->replica_rows(rep, &n_cv, &ran, err);
  if (rc) return rc;
  bool any_cv = false;
  for (uint32_t c = 0; c < ncol; c++) {
    if (species[c] >= nsp || !names[c] || objects[c] < -1 || (objects[c] >= 0 && (uint32_t)objects[c] >= n_cv)) {
      err = "count column " + std::to_string(c) + ": species or counted object out of range";
      return MCG_ERR_ARG;
    }
    any_cv = any_cv || objects[c] >= 0;
  }
  if (n_it > ran) {
    err = "mcg_write_counts: more rows asked for than iterations run";
    return MCG_ERR_ARG;
  }
  std::vector<uint64_t> world((size_t)n_it * nsp), inside;
  if (n_it) {
    rc = dev->trajectory(rep, n_it, world.data(), err);
    if (rc) return rc;
    if (any_cv) {
      inside.resize((size_t)n_it * nsp * n_cv);
      rc = dev->counted_trajectory(rep, n_it, inside.data(), err);
      if (rc) return rc;
    }
  }
  std::vector<uint32_t> rows;
  std::vector<double> times;
  // a window that reaches back to the replica's start begins with the counts before
  // its first iteration, at t = 0, as the reference's count event runs before the
  // diffusion event in iteration 0 (row index n_it stands for it)
  std::vector<uint64_t> world0(nsp), inside0((size_t)nsp * n_cv);
  const bool row0 = n_it == ran && dev->initial_counts(rep, world0.data(), inside0.data(), err) == 0;
  err.clear();
  if (row0) {
    rows.push_back(n_it);
    times.push_back(0.0);
  }
  auto value = [&](uint32_t k, uint32_t c) -> double {
    if (k == n_it) return (double)(objects[c] < 0 ? world0[species[c]] : inside0[(size_t)species[c] * n_cv + (uint32_t)objects[c]]);
    if (objects[c] < 0) return (double)world[(size_t)k * nsp + species[c]];
    return (double)inside[((size_t)k * nsp + species[c]) * n_cv + (uint32_t)objects[c]];
  };
  for (uint32_t k = 0; k < n_it; k++) {
    const uint64_t it = ran - n_it + k + 1;  // iterations run after row k
    if (it % every) continue;
    rows.push_back(k);
    times.push_back((double)it * dt);
  }
  auto open = [&](const std::string& path, std::ofstream& f) -> bool {
    std::error_code ec;
    const std::filesystem::path parent = std::filesystem::path(path).parent_path();
    if (!parent.empty()) std::filesystem::create_directories(parent, ec);
    f.open(path);
    if (!f) err = "cannot open " + path;
    return (bool)f;
  };
  if (format == MCG_COUNTS_DAT) {
    for (uint32_t c = 0; c < ncol; c++) {
      std::ofstream f;
      const std::string path = std::string(prefix) + "." + names[c] + ".dat";
      if (!open(path, f)) return MCG_ERR_ARG;
      for (size_t r = 0; r < rows.size(); r++) f << times[r] << " " << value(rows[r], c) << "\n";
      if (!f) {
        err = "writing " + path + " failed";
        return MCG_ERR_ARG;
      }
    }
    return MCG_OK;
  }
  std::ofstream f;
  const std::string path = std::string(prefix) + ".gdat";
  if (!open(path, f)) return MCG_ERR_ARG;
  // header (CountBuffer::write_gdat_header): '#', "time" and the names right-aligned
  std::string t = "time";
  t.insert(t.begin(), 14 - t.size(), ' ');
  f << "#" << t;
  for (uint32_t c = 0; c < ncol; c++) {
    std::string col = names[c];
    if (14 > col.size())
      col.insert(col.begin(), 14 - col.size() + 2, ' ');
    else
      col = " " + col;
    f << col;
  }
  f << "\n";
  for (size_t r = 0; r < rows.size(); r++) {
    f << " " << gdat_number(times[r]);
    for (uint32_t c = 0; c < ncol; c++) f << "  " << gdat_number(value(rows[r], c));
    f << "\n";
  }
  if (!f) {
    err = "writing " + path + " failed";
    return MCG_ERR_ARG;
  }
  return MCG_OK;
}

}  // namespace

extern "C" {

int mcg_write_counts(mcg_engine* e, const char* prefix, int format, uint32_t n_iterations, uint32_t every,
                     double time_step_s, uint32_t n_columns, const uint32_t* species, const int32_t* objects,
                     const char* const* names) {
  if (!e || !prefix) return MCG_ERR_ARG;
  if (!e->dev) {
    e->err = "mcg_write_counts needs a prepared engine";
    return MCG_ERR_ARG;
  }
  std::string err;
  int rc = write_counts(e->dev, 0, e->cfg.n_species, prefix, format, n_iterations, every, time_step_s, n_columns,
                        species, objects, names, err);
  if (rc) e->err = err;
  return rc;
}


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

int mcg_batch_write_counts(mcg_batch* b, uint32_t replica, const char* prefix, int format, uint32_t n_iterations,
                           uint32_t every, double time_step_s, uint32_t n_columns, const uint32_t* species,
                           const int32_t* objects, const char* const* names) {
  if (!b || !prefix) return MCG_ERR_ARG;
  if (!b->dev) {
    b->err = "batch has no device engine";
    return MCG_ERR_CUDA;
  }
  std::string err;
  int rc = write_counts(b->dev, replica, b->cfg.n_species, prefix, format, n_iterations, every, time_step_s, n_columns,
                        species, objects, names, err);
  if (rc) b->err = err;
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
