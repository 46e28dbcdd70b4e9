// fv_ini.cpp -- the reference's .ini configuration surface.
//
// fv_read_ini / fv_parse_ini reproduce fv3d::readInifile (SimInfo.h:169-306):
// the same sections, keys, defaults, derived mesh quantities and the
// std::map::operator[] fallback that turns an unknown enum string into value 0.
// The parser follows the jtilly/inih INIReader the reference includes
// (SimInfo.h:5): case-insensitive section/key names, case-sensitive values,
// ';'/'#' comment lines, ';' inline comments after whitespace, '=' or ':'
// separators, indented continuation lines, repeated keys joined by "\n";
// GetInteger parses with strtol(base 0), GetFloat with strtof -- so every
// GetFloat setting (gamma0, CFL, tend, xmin, ...) carries single precision,
// exactly as in the reference -- and GetBoolean accepts true/yes/on/1 and
// false/no/off/0.
#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>

#include "fv3d_gb300.h"

namespace {

class IniValues {
 public:
  explicit IniValues(const std::string& text) { Parse(text); }

  std::string Get(const std::string& section, const std::string& name, const std::string& dflt) const {
    auto it = values_.find(Key(section, name));
    return it == values_.end() ? dflt : it->second;
  }
  long GetInteger(const std::string& section, const std::string& name, long dflt) const {
    const std::string v = Get(section, name, "");
    char* end = nullptr;
    const long n = std::strtol(v.c_str(), &end, 0);
    return end > v.c_str() ? n : dflt;
  }
  float GetFloat(const std::string& section, const std::string& name, float dflt) const {
    const std::string v = Get(section, name, "");
    char* end = nullptr;
    const float n = std::strtof(v.c_str(), &end);
    return end > v.c_str() ? n : dflt;
  }
  bool GetBoolean(const std::string& section, const std::string& name, bool dflt) const {
    std::string v = Get(section, name, "");
    for (char& c : v) c = (char)std::tolower((unsigned char)c);
    if (v == "true" || v == "yes" || v == "on" || v == "1") return true;
    if (v == "false" || v == "no" || v == "off" || v == "0") return false;
    return dflt;
  }

 private:
  static std::string Lower(std::string s) {
    for (char& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
  }
  static std::string Key(const std::string& section, const std::string& name) {
    return Lower(section + "=" + name);
  }
  static bool Space(char c) { return std::isspace((unsigned char)c) != 0; }
  static std::string Trim(const std::string& s, size_t b, size_t e) {
    while (b < e && Space(s[b])) ++b;
    while (e > b && Space(s[e - 1])) --e;
    return s.substr(b, e - b);
  }
  // First position of one of `stops` or of a ';' that follows whitespace.
  static size_t Scan(const std::string& s, size_t p, const char* stops) {
    bool prev_space = false;
    for (; p < s.size(); ++p) {
      const char c = s[p];
      if (stops && c != '\0' && std::strchr(stops, c)) return p;
      if (prev_space && c == ';') return p;
      prev_space = Space(c);
    }
    return s.size();
  }
  void Add(const std::string& section, const std::string& name, const std::string& value) {
    std::string& slot = values_[Key(section, name)];
    if (!slot.empty()) slot += "\n";
    slot += value;
  }
  void Parse(const std::string& text) {
    std::string section, last_name;
    size_t pos = 0;
    bool first = true;
    while (pos < text.size()) {
      size_t nl = text.find('\n', pos);
      if (nl == std::string::npos) nl = text.size();
      std::string line = text.substr(pos, nl - pos);
      pos = nl + 1;
      if (first && line.size() >= 3 && (unsigned char)line[0] == 0xEF && (unsigned char)line[1] == 0xBB &&
          (unsigned char)line[2] == 0xBF)
        line.erase(0, 3);
      first = false;
      size_t e = line.size();
      while (e > 0 && Space(line[e - 1])) --e;
      size_t b = 0;
      while (b < e && Space(line[b])) ++b;
      if (b == e) continue;
      if (line[b] == ';' || line[b] == '#') continue;
      if (b > 0 && !last_name.empty()) {  // indented: continuation of the last value
        Add(section, last_name, line.substr(b, e - b));
        continue;
      }
      const std::string body = line.substr(0, e);
      if (body[b] == '[') {
        const size_t close = Scan(body, b + 1, "]");
        if (close < body.size() && body[close] == ']') {
          section = body.substr(b + 1, close - b - 1);
          last_name.clear();
        }
        continue;
      }
      const size_t sep = Scan(body, b, "=:");
      if (sep < body.size() && (body[sep] == '=' || body[sep] == ':')) {
        const std::string name = Trim(body, b, sep);
        size_t vb = sep + 1;
        while (vb < body.size() && Space(body[vb])) ++vb;
        const size_t ve = Scan(body, vb, nullptr);
        const std::string value = Trim(body, vb, ve);
        last_name = name;
        Add(section, name, value);
      }
    }
  }

  std::map<std::string, std::string> values_;
};

template <class E>
int Lookup(const std::map<std::string, E>& m, const std::string& key) {
  auto it = m.find(key);
  return it == m.end() ? 0 : (int)it->second;  // std::map::operator[] default
}

void FromValues(const IniValues& r, fv_params* o) {
  std::memset(o, 0, sizeof(*o));
  o->Nx = (int)r.GetInteger("mesh", "Nx", 32);
  o->Ny = (int)r.GetInteger("mesh", "Ny", 32);
  o->Nz = (int)r.GetInteger("mesh", "Nz", 32);
  o->Ng = (int)r.GetInteger("mesh", "Nghosts", 2);
  o->xmin = r.GetFloat("mesh", "xmin", 0.0);
  o->xmax = r.GetFloat("mesh", "xmax", 1.0);
  o->ymin = r.GetFloat("mesh", "ymin", 0.0);
  o->ymax = r.GetFloat("mesh", "ymax", 1.0);
  o->zmin = r.GetFloat("mesh", "zmin", 0.0);
  o->zmax = r.GetFloat("mesh", "zmax", 1.0);
  o->dx = (o->xmax - o->xmin) / o->Nx;
  o->dy = (o->ymax - o->ymin) / o->Ny;
  o->dz = (o->zmax - o->zmin) / o->Nz;

  o->tend = r.GetFloat("run", "tend", 1.0);
  o->save_freq = r.GetFloat("run", "save_freq", 1.0e-1);
  std::strncpy(o->filename_out, r.Get("run", "output_filename", "run").c_str(), sizeof(o->filename_out) - 1);

  const std::map<std::string, int> bc{{"reflecting", FV_BC_REFLECTING},
                                      {"absorbing", FV_BC_ABSORBING},
                                      {"periodic", FV_BC_PERIODIC},
                                      {"C91", FV_BC_C91}};
  o->boundary_x = Lookup(bc, r.Get("run", "boundaries_x", "reflecting"));
  o->boundary_y = Lookup(bc, r.Get("run", "boundaries_y", "reflecting"));
  o->boundary_z = Lookup(bc, r.Get("run", "boundaries_z", "reflecting"));

  const std::map<std::string, int> recon{{"pcm", FV_PCM}, {"pcm_wb", FV_PCM_WB}, {"plm", FV_PLM}};
  o->reconstruction = Lookup(recon, r.Get("solvers", "reconstruction", "pcm"));
  const std::map<std::string, int> rs{{"hll", FV_HLL}, {"hllc", FV_HLLC}};
  o->riemann_solver = Lookup(rs, r.Get("solvers", "riemann_solver", "hllc"));
  const std::map<std::string, int> ts{{"euler", FV_TS_EULER}, {"RK2", FV_TS_RK2}};
  o->time_stepping = Lookup(ts, r.Get("solvers", "time_stepping", "euler"));
  o->CFL = r.GetFloat("solvers", "CFL", 0.8);

  o->epsilon = r.GetFloat("misc", "epsilon", 1.0e-6);
  o->gamma0 = r.GetFloat("physics", "gamma0", 5.0 / 3.0);
  o->gravity = r.GetBoolean("physics", "gravity", false);
  o->g = r.GetFloat("physics", "g", 0.0);
  o->m1 = r.GetFloat("polytrope", "m1", 1.0);
  o->theta1 = r.GetFloat("polytrope", "theta1", 10.0);
  o->m2 = r.GetFloat("polytrope", "m2", 1.0);
  o->theta2 = r.GetFloat("polytrope", "theta2", 10.0);
  std::strncpy(o->problem, r.Get("physics", "problem", "blast").c_str(), sizeof(o->problem) - 1);
  o->well_balanced_flux_at_z_bc = r.GetBoolean("physics", "well_balanced_flux_at_z_bc", false);

  o->thermal_conductivity_active = r.GetBoolean("thermal_conduction", "active", false);
  const std::map<std::string, int> tcm{{"constant", FV_TCM_CONSTANT}, {"B02", FV_TCM_B02}};
  o->thermal_conductivity_mode = Lookup(tcm, r.Get("thermal_conduction", "conductivity_mode", "constant"));
  o->kappa = r.GetFloat("thermal_conduction", "kappa", 0.0);
  const std::map<std::string, int> bctc{{"none", FV_BCTC_NONE},
                                        {"fixed_temperature", FV_BCTC_FIXED_TEMPERATURE},
                                        {"fixed_gradient", FV_BCTC_FIXED_GRADIENT}};
  o->bctc_zmin = Lookup(bctc, r.Get("thermal_conduction", "bc_zmin", "none"));
  o->bctc_zmax = Lookup(bctc, r.Get("thermal_conduction", "bc_zmax", "none"));
  o->bctc_zmin_value = r.GetFloat("thermal_conduction", "bc_zmin_value", 1.0);
  o->bctc_zmax_value = r.GetFloat("thermal_conduction", "bc_zmax_value", 1.0);

  o->viscosity_active = r.GetBoolean("viscosity", "active", false);
  const std::map<std::string, int> vm{{"constant", FV_VSC_CONSTANT}};
  o->viscosity_mode = Lookup(vm, r.Get("viscosity", "viscosity_mode", "constant"));
  o->mu = r.GetFloat("viscosity", "mu", 0.0);

  o->h84_pert = r.GetFloat("H84", "perturbation", 1.0e-4);
  o->c91_pert = r.GetFloat("C91", "perturbation", 1.0e-3);
  o->seed = (int)r.GetInteger("misc", "seed", 12345);
  o->log_frequency = (int)r.GetInteger("misc", "log_frequency", 10);

  // Driver-only key (no reference counterpart): storage/arithmetic of the GPU path.
  const std::map<std::string, int> prec{{"fp64", FV_PREC_FP64}, {"fp32_mixed", FV_PREC_FP32_MIXED}};
  o->precision = Lookup(prec, r.Get("gpu", "precision", "fp64"));
  const std::map<std::string, int> phys{{"reference", FV_PHYS_REFERENCE}, {"corrected", FV_PHYS_CORRECTED}};
  o->physics = Lookup(phys, r.Get("gpu", "physics", "reference"));
}

}  // namespace

extern "C" {

const char* fv_status_string(int status) {
  switch (status) {
    case FV_OK: return "FV_OK";
    case FV_ERR_PARAM: return "FV_ERR_PARAM";
    case FV_ERR_UNSUPPORTED: return "FV_ERR_UNSUPPORTED";
    case FV_ERR_CUDA: return "FV_ERR_CUDA";
    case FV_ERR_NONFINITE: return "FV_ERR_NONFINITE";
    case FV_ERR_NOMEM: return "FV_ERR_NOMEM";
    case FV_ERR_IO: return "FV_ERR_IO";
    case FV_ERR_TIMEOUT: return "FV_ERR_TIMEOUT";
    case FV_ERR_STATE: return "FV_ERR_STATE";
    default: return "FV_ERR_UNKNOWN";
  }
}

int fv_parse_ini(const char* text, fv_params* out) {
  if (!text || !out) return FV_ERR_PARAM;
  FromValues(IniValues(text), out);
  return FV_OK;
}

int fv_read_ini(const char* path, fv_params* out) {
  if (!path || !out) return FV_ERR_PARAM;
  std::ifstream in(path, std::ios::binary);
  std::string text;
  if (in) {  // like the reference, an unreadable file leaves every default
    std::stringstream ss;
    ss << in.rdbuf();
    text = ss.str();
  }
  FromValues(IniValues(text), out);
  return FV_OK;
}

}  // extern "C"
