// e2d_config.cpp -- the reference's parameter contract on the host:
// an ini reader with the reading rules of the reference's ConfigMap
// (config/ConfigMap.{h,cpp} over config/inih) and HydroParams::setup / init
// (src/HydroParams.cpp:42-190) filling the flat e2d_params of include/e2d.h.
//
// Reading rules, each of which changes parsed values (restated from the
// behaviour of config/inih/ini.cpp:66-150 and config/inih/INIReader.cpp):
//  R1 the file is consumed in records of at most 199 bytes: a record ends
//     after a '\n' or once 199 bytes are read (a longer line continues as the
//     next record); records are numbered from 1; a NUL byte ends a record's text;
//  R2 each record is trimmed of whitespace (isspace) at both ends;
//  R3 a record that began with whitespace and is not blank, read while a key
//     is current, replaces that key's value (no comment rule applies to it);
//  R4 a record starting with ';' or '#' is a comment;
//  R5 '[' opens a section name closed by the first ']'; a ';' right after a
//     whitespace character ends the search (no ']': an error); the name
//     keeps at most 49 bytes; afterwards no key is current;
//  R6 any other record is name '=' value, split at the first '=' met before
//     a whitespace-preceded ';' (none: an error); the name is right-trimmed,
//     the value left-trimmed, cut at its first whitespace-preceded ';' and
//     right-trimmed; the key becomes current, its name kept to 49 bytes;
//  R7 keys are "section.name" lower-cased; a later value replaces an earlier;
//  R8 parsing always reads to the end; the result is 0 or the number of the
//     first record in error;
// and, for values:
//  - reals are parsed with strtof and returned as float, so gamma0=1.4 is
//    really (double)1.4f (config/ConfigMap.cpp:31-40), defaults included;
//  - integers use strtol base 0 ("010" is 8; config/inih/INIReader.cpp:57-66).
#include "e2d_internal.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace e2d {

namespace {

constexpr size_t kRecordBytes = 199;  // R1
constexpr size_t kNameBytes = 49;     // R5, R6

bool is_ws(char c) { return std::isspace(static_cast<unsigned char>(c)) != 0; }

// R5/R6: index of the first `stop` in text[from, to), or of a ';' whose
// preceding character (within the scanned range) is whitespace, else `to`.
size_t scan(const std::string &text, size_t from, size_t to, char stop) {
  for (size_t k = from; k < to; ++k) {
    if (text[k] == stop) return k;
    if (text[k] == ';' && k > from && is_ws(text[k - 1])) return k;
  }
  return to;
}

size_t trim_right(const std::string &text, size_t from, size_t to) {
  while (to > from && is_ws(text[to - 1])) --to;
  return to;
}

std::string make_key(const std::string &section, const std::string &name) {  // R7
  std::string key = section + "." + name;
  for (auto &ch : key) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  return key;
}

// R1: the records of a file.
bool read_records(const char *path, std::vector<std::string> *records) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  std::string rec;
  int ch;
  while ((ch = std::fgetc(f)) != EOF) {
    rec.push_back(static_cast<char>(ch));
    if (ch == '\n' || rec.size() == kRecordBytes) {
      records->push_back(rec);
      rec.clear();
    }
  }
  if (!rec.empty()) records->push_back(rec);
  std::fclose(f);
  for (auto &r : *records) {
    const size_t nul = r.find('\0');
    if (nul != std::string::npos) r.resize(nul);
  }
  return true;
}

}  // namespace

int IniMap::parse(const char *path) {
  std::vector<std::string> records;
  if (!read_records(path, &records)) return -1;
  std::string section, current;  // current: name of the key R3 continues
  int first_error = 0;
  auto fail = [&](int number) {
    if (!first_error) first_error = number;
  };
  for (size_t r = 0; r < records.size(); ++r) {
    const std::string &text = records[r];
    const int number = static_cast<int>(r) + 1;
    const size_t end = trim_right(text, 0, text.size());  // R2
    size_t begin = 0;
    while (begin < end && is_ws(text[begin])) ++begin;
    if (begin == end) continue;  // blank
    const char lead = text[begin];
    if (begin > 0 && !current.empty()) {  // R3
      values_[make_key(section, current)] = text.substr(begin, end - begin);
    } else if (lead == ';' || lead == '#') {  // R4
    } else if (lead == '[') {  // R5
      const size_t close = scan(text, begin + 1, end, ']');
      if (close < end && text[close] == ']') {
        section = text.substr(begin + 1, std::min(close - begin - 1, kNameBytes));
        current.clear();
      } else {
        fail(number);
      }
    } else {  // R6
      const size_t eq = scan(text, begin, end, '=');
      if (eq < end && text[eq] == '=') {
        const std::string name = text.substr(begin, trim_right(text, begin, eq) - begin);
        size_t vb = eq + 1;
        while (vb < end && is_ws(text[vb])) ++vb;
        const size_t ve = trim_right(text, vb, scan(text, vb, end, '\0'));
        values_[make_key(section, name)] = text.substr(vb, ve - vb);
        current = name.substr(0, kNameBytes);
      } else {
        fail(number);
      }
    }
  }
  return first_error;  // R8
}

std::string IniMap::get_string(const std::string &section, const std::string &name,
                               const std::string &dflt) const {
  auto it = values_.find(make_key(section, name));
  return it == values_.end() ? dflt : it->second;
}

long IniMap::get_integer(const std::string &section, const std::string &name, long dflt) const {
  std::string s = get_string(section, name, "");
  const char *v = s.c_str();
  char *end = nullptr;
  long n = std::strtol(v, &end, 0);
  return end > v ? n : dflt;
}

float IniMap::get_float(const std::string &section, const std::string &name, float dflt) const {
  std::string s = get_string(section, name, "");
  const char *v = s.c_str();
  char *end = nullptr;
  float x = std::strtof(v, &end);
  return end > v ? x : dflt;
}

bool IniMap::get_bool(const std::string &section, const std::string &name, bool dflt) const {
  std::string s = get_string(section, name, "");
  bool val = dflt;
  if (s == "1" || s == "yes" || s == "true" || s == "on") val = true;
  if (s == "0" || s == "no" || s == "false" || s == "off") val = false;
  if (s.empty()) val = dflt;
  return val;
}

// HydroParams() member defaults (src/HydroParams.h:222-258) and the
// defaults HydroParams::setup passes to ConfigMap (src/HydroParams.cpp).
void params_defaults(e2d_params *p) {
  std::memset(p, 0, sizeof(*p));
  p->nStepmax = 1000;
  p->tEnd = 0.0;
  p->nOutput = 100;
  p->enableOutput = 1;
  p->ioVTK = 1;
  p->ioHDF5 = 0;
  p->blast_nbins = 100;
  p->nx = 2;
  p->ny = 2;
  p->ghostWidth = 2;
  p->xmin = 0.0;
  p->xmax = 1.0;
  p->ymin = 0.0;
  p->ymax = 1.0;
  p->boundary_type_xmin = p->boundary_type_xmax = E2D_BC_REFLECT;
  p->boundary_type_ymin = p->boundary_type_ymax = E2D_BC_REFLECT;
  p->gamma0 = (double)1.4f;
  p->cfl = (double)0.5f;
  p->slope_type = 1.0;
  p->smallr = (double)1e-10f;
  p->smallc = (double)1e-10f;
  p->niter_riemann = 10;
  p->riemannSolverType = E2D_RIEMANN_APPROX;
  p->problemType = E2D_PROBLEM_IMPLODE;
  p->blast_radius = (double)(float)(1.0 / 2.0 / 10);
  p->blast_center_x = (double)0.5f;
  p->blast_center_y = (double)0.5f;
  p->blast_density_in = 1.0;
  p->blast_density_out = (double)1.2f;
  p->blast_pressure_in = 10.0;
  p->blast_pressure_out = (double)0.1f;
  p->blast_total_energy_inside = 0.0;
  p->bubble_radius = (double)0.025f;
  p->bubble_center_x = (double)0.225f;
  p->bubble_center_y = (double)0.0445f;
  p->bubble_density = (double)3.863f;
  p->bubble_pressure = (double)1.0132e5f;
  p->preshock_density = (double)1.225f;
  p->preshock_pressure = (double)1.0132e5f;
  p->postshock_density = (double)1.686f;
  p->postshock_pressure = (double)1.59e5f;
  p->postshock_velocity = (double)113.5f;
  p->shock_loc = (double)0.170f;
  // src/HydroRunFunctors.h:1607-1622: real_t literals, not ini reals
  p->fq_split_x = 0.8;
  p->fq_split_y = 0.8;
  static const double lax_liu_3[4][4] = {
      {1.5, 1.5, 0.0, 0.0}, {0.5323, 0.3, 1.206, 0.0}, {0.138, 0.029, 1.206, 1.206}, {0.5323, 0.3, 0.0, 1.206}};
  std::memcpy(p->fq_state, lax_liu_3, sizeof(lax_liu_3));
  p->implode_shape = 0;
  p->implementationVersion = 0;
  p->precision = E2D_PRECISION_FP64;
}

// src/HydroParams.cpp:42-156 (HydroParams::setup), then init().
int params_from_ini(const IniMap &m, e2d_params *p, std::string *msg) {
  params_defaults(p);
  p->nStepmax = (int)m.get_integer("run", "nstepmax", 1000);
  p->tEnd = m.get_float("run", "tend", 0.0f);
  p->nOutput = (int)m.get_integer("run", "noutput", 100);
  p->enableOutput = (p->nOutput == -1) ? 0 : 1;
  // the defaults of a build without HDF5 (src/HydroParams.cpp:54-60)
  p->ioHDF5 = m.get_bool("run", "use_HDF5", false) ? 1 : 0;
  p->ioVTK = m.get_bool("run", "use_VTK", true) ? 1 : 0;

  p->nx = (int)m.get_integer("mesh", "nx", 2);
  p->ny = (int)m.get_integer("mesh", "ny", 2);
  p->xmin = m.get_float("mesh", "xmin", 0.0f);
  p->ymin = m.get_float("mesh", "ymin", 0.0f);
  p->xmax = m.get_float("mesh", "xmax", 1.0f);
  p->ymax = m.get_float("mesh", "ymax", 1.0f);
  p->boundary_type_xmin = (int)m.get_integer("mesh", "boundary_type_xmin", E2D_BC_REFLECT);
  p->boundary_type_xmax = (int)m.get_integer("mesh", "boundary_type_xmax", E2D_BC_REFLECT);
  p->boundary_type_ymin = (int)m.get_integer("mesh", "boundary_type_ymin", E2D_BC_REFLECT);
  p->boundary_type_ymax = (int)m.get_integer("mesh", "boundary_type_ymax", E2D_BC_REFLECT);

  p->gamma0 = m.get_float("hydro", "gamma0", 1.4f);
  p->cfl = m.get_float("hydro", "cfl", 0.5f);
  p->slope_type = m.get_float("hydro", "slope_type", 1.0f);
  p->smallc = m.get_float("hydro", "smallc", 1e-10f);
  p->smallr = m.get_float("hydro", "smallr", 1e-10f);
  p->niter_riemann = (int)m.get_integer("hydro", "niter_riemann", 10);

  const std::string rs = m.get_string("hydro", "riemann", "approx");
  if (rs == "approx")
    p->riemannSolverType = E2D_RIEMANN_APPROX;
  else if (rs == "hll")
    p->riemannSolverType = E2D_RIEMANN_HLL;
  else if (rs == "hllc")
    p->riemannSolverType = E2D_RIEMANN_HLLC;
  else {
    // the reference prints a notice and falls back to approx (:100-105)
    p->riemannSolverType = E2D_RIEMANN_APPROX;
    if (msg) *msg += "riemann solver '" + rs + "' is invalid, using approx; ";
  }

  const std::string ps = m.get_string("hydro", "problem", "unknown");
  if (ps == "implode")
    p->problemType = E2D_PROBLEM_IMPLODE;
  else if (ps == "blast")
    p->problemType = E2D_PROBLEM_BLAST;
  else if (ps == "four_quadrant")
    p->problemType = E2D_PROBLEM_FOUR_QUADRANT;
  else if (ps == "discontinuity")
    p->problemType = E2D_PROBLEM_DISCONTINUITY;
  else if (ps == "shocked_bubble")
    p->problemType = E2D_PROBLEM_SHOCKED_BUBBLE;
  else {
    p->problemType = E2D_PROBLEM_IMPLODE;
    if (msg) *msg += "problem '" + ps + "' is invalid, using implode; ";
  }

  // src/HydroParams.cpp:19-37 (readShockedBubbleParams)
  p->bubble_radius = m.get_float("shocked_bubble", "bubble_radius", 0.025f);
  p->bubble_center_x = m.get_float("shocked_bubble", "bubble_center_x", 0.225f);
  p->bubble_center_y = m.get_float("shocked_bubble", "bubble_center_y", 0.0445f);
  p->bubble_density = m.get_float("shocked_bubble", "bubble_density", 3.863f);
  p->bubble_pressure = m.get_float("shocked_bubble", "bubble_pressure", 1.0132e5f);
  p->preshock_density = m.get_float("shocked_bubble", "preshock_density", 1.225f);
  p->preshock_pressure = m.get_float("shocked_bubble", "preshock_pressure", 1.0132e5f);
  p->postshock_density = m.get_float("shocked_bubble", "postshock_density", 1.686f);
  p->postshock_pressure = m.get_float("shocked_bubble", "postshock_pressure", 1.59e5f);
  p->postshock_velocity = m.get_float("shocked_bubble", "postshock_velocity", 113.5f);
  p->shock_loc = m.get_float("shocked_bubble", "shock_loc", 0.170f);

  // defaults depend on the mesh, computed in double then narrowed to float
  p->blast_radius = m.get_float("blast", "radius", (float)((p->xmin + p->xmax) / 2.0 / 10));
  p->blast_center_x = m.get_float("blast", "center_x", (float)((p->xmin + p->xmax) / 2));
  p->blast_center_y = m.get_float("blast", "center_y", (float)((p->ymin + p->ymax) / 2));
  p->blast_density_in = m.get_float("blast", "density_in", 1.0f);
  p->blast_density_out = m.get_float("blast", "density_out", 1.2f);
  p->blast_pressure_in = m.get_float("blast", "pressure_in", 10.0f);
  p->blast_pressure_out = m.get_float("blast", "pressure_out", 0.1f);
  p->blast_total_energy_inside = m.get_float("blast", "total_energy_inside", 0.0f);
  p->blast_nbins = (int)m.get_integer("blast", "nbins", 100);

  // extension keys (absent keys keep the reference's behaviour)
  const std::string none = "\x01";
  auto opt_float = [&](const char *sec, const std::string &key, double dflt) {
    return m.get_string(sec, key, none) == none ? dflt : (double)m.get_float(sec, key, 0.0f);
  };
  p->fq_split_x = opt_float("four_quadrant", "split_x", p->fq_split_x);
  p->fq_split_y = opt_float("four_quadrant", "split_y", p->fq_split_y);
  static const char *const fq_names[4] = {"rho_", "p_", "u_", "v_"};
  for (int q = 0; q < 4; ++q)
    for (int v = 0; v < 4; ++v)
      p->fq_state[q][v] = opt_float("four_quadrant", fq_names[v] + std::to_string(q), p->fq_state[q][v]);
  p->implode_shape = (int)m.get_integer("implode", "shape", 0);
  const std::string prec = m.get_string("gb300", "precision", "fp64");
  p->precision = (prec == "fp32c") ? E2D_PRECISION_FP32C
                  : (prec == "fp64_fast") ? E2D_PRECISION_FP64_FAST : E2D_PRECISION_FP64;

  // getFloat then an implicit float->int conversion (:149-155)
  p->implementationVersion = (int)m.get_float("OTHER", "implementationVersion", 0.0f);
  if (p->implementationVersion != 0 && p->implementationVersion != 1 &&
      p->implementationVersion != 2) {
    if (msg) *msg += "implementation version is invalid, using 0; ";
    p->implementationVersion = 0;
  }
  return params_init(p, msg);
}

// src/HydroParams.cpp:160-190 (HydroParams::init) plus the validation the
// GPU path needs (the reference exits or runs undefined code on these).
int params_init(e2d_params *p, std::string *msg) {
  if (p->ghostWidth != 2) {
    if (msg) *msg += "ghostWidth must be 2; ";
    return E2D_EINVAL;
  }
  p->imin = 0;
  p->jmin = 0;
  p->imax = p->nx - 1 + 2 * p->ghostWidth;
  p->jmax = p->ny - 1 + 2 * p->ghostWidth;
  p->isize = p->imax - p->imin + 1;
  p->jsize = p->jmax - p->jmin + 1;
  p->dx = (p->xmax - p->xmin) / p->nx;
  p->dy = (p->ymax - p->ymin) / p->ny;
  p->smallp = p->smallc * p->smallc / p->gamma0;
  p->smallpp = p->smallr * p->smallp;
  p->gamma6 = (p->gamma0 + 1.0) / (2.0 * p->gamma0);

  auto bad = [&](const char *what) {
    if (msg) *msg += std::string(what) + "; ";
    return E2D_EINVAL;
  };
  if (p->nx < 1 || p->ny < 1) return bad("nx and ny must be >= 1");
  if ((long long)p->isize * p->jsize >= (1LL << 31)) return bad("grid too large (isize*jsize >= 2^31)");
  const int bcs[4] = {p->boundary_type_xmin, p->boundary_type_xmax, p->boundary_type_ymin,
                      p->boundary_type_ymax};
  for (int b : bcs)
    if (b < E2D_BC_REFLECT || b > E2D_BC_PERIODIC) return bad("boundary_type must be 1, 2 or 3");
  // every ghost cell must take its value from an interior cell, which needs
  // an interior at least as wide as the ghost layer
  if (p->nx < 2 || p->ny < 2) return bad("nx and ny must be >= 2 (ghost layer of 2)");
  if (!(p->slope_type == 0.0 || p->slope_type == 1.0 || p->slope_type == 2.0))
    return bad("slope_type must be 0, 1 or 2");
  if (!(p->gamma0 > 1.0)) return bad("gamma0 must be > 1");
  if (!(p->cfl > 0.0)) return bad("cfl must be > 0");
  if (!(p->dx > 0.0) || !(p->dy > 0.0)) return bad("xmax > xmin and ymax > ymin required");
  if (!(p->smallr > 0.0) || !(p->smallc > 0.0)) return bad("smallr and smallc must be > 0");
  if (p->riemannSolverType < 0 || p->riemannSolverType > 2) return bad("riemann solver must be 0, 1 or 2");
  if (p->precision != E2D_PRECISION_FP64 && p->precision != E2D_PRECISION_FP32C &&
      p->precision != E2D_PRECISION_FP64_FAST)
    return bad("precision must be fp64, fp32c or fp64_fast");
  if (p->problemType < 0 || p->problemType > 4) return bad("problem must be 0..4");
  return E2D_OK;
}

}  // namespace e2d
