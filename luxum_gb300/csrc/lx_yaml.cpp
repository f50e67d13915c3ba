// lx_yaml.cpp -- reader for Luxum's parameters.yaml (reader::readYAML, reader.cc:68-130).
//
// The file is a UTF-8 (optionally BOM-prefixed) stream of five flow mappings, one per YAML
// document, with quoted keys, '#' comments and trailing commas (parameters.yaml:1-59).  The
// reference reads it with yaml-cpp 0.3 (GetNextDocument + operator>>); this parser accepts
// exactly that shape: a sequence of "{ key: scalar, ... }" blocks, optional "---" markers.
// A sixth mapping, when present, carries engine options the reference hard-codes.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "luxum.h"

namespace lx {
lx_status set_thread_error(const char* msg, lx_status st);
}
using lx::set_thread_error;

namespace {

using Doc = std::map<std::string, std::string>;

struct Parser {
  const std::string& s;
  size_t i = 0;
  std::string err;
  explicit Parser(const std::string& src) : s(src) {}

  void skip_ws() {
    for (;;) {
      while (i < s.size() && (std::isspace((unsigned char)s[i]) || s[i] == ',')) i++;
      if (i < s.size() && s[i] == '#') {
        while (i < s.size() && s[i] != '\n') i++;
        continue;
      }
      if (s.compare(i, 3, "\xEF\xBB\xBF") == 0) {  // BOM (parameters.yaml:1)
        i += 3;
        continue;
      }
      if (s.compare(i, 3, "---") == 0 || s.compare(i, 3, "...") == 0) {
        i += 3;
        continue;
      }
      break;
    }
  }

  bool scalar(std::string& out, bool is_key) {
    skip_inline();
    if (i >= s.size()) return false;
    char q = s[i];
    if (q == '"' || q == '\'') {
      i++;
      out.clear();
      while (i < s.size() && s[i] != q) {
        if (q == '"' && s[i] == '\\' && i + 1 < s.size()) i++;
        out += s[i++];
      }
      if (i >= s.size()) { err = "unterminated quoted scalar"; return false; }
      i++;
      return true;
    }
    size_t b = i;
    while (i < s.size()) {
      char ch = s[i];
      if (ch == ',' || ch == '}' || ch == '\n' || ch == '#') break;
      if (is_key && ch == ':') break;
      i++;
    }
    out = s.substr(b, i - b);
    while (!out.empty() && std::isspace((unsigned char)out.back())) out.pop_back();
    return !out.empty();
  }

  void skip_inline() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r' || s[i] == '\n')) i++;
    while (i < s.size() && s[i] == '#') {
      while (i < s.size() && s[i] != '\n') i++;
      while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
    }
  }

  bool mapping(Doc& d) {
    skip_ws();
    if (i >= s.size()) return false;
    if (s[i] != '{') { err = "expected '{' at offset " + std::to_string(i); return false; }
    i++;
    for (;;) {
      skip_ws();
      if (i >= s.size()) { err = "unterminated mapping"; return false; }
      if (s[i] == '}') { i++; return true; }
      std::string k, v;
      if (!scalar(k, true)) { if (err.empty()) err = "expected key"; return false; }
      skip_inline();
      if (i >= s.size() || s[i] != ':') { err = "expected ':' after key \"" + k + "\""; return false; }
      i++;
      if (!scalar(v, false)) { if (err.empty()) err = "expected value for key \"" + k + "\""; return false; }
      d[k] = v;
    }
  }
};

bool to_bool(const std::string& v, int& out) {
  std::string l;
  for (char ch : v) l += (char)std::tolower((unsigned char)ch);
  if (l == "true" || l == "yes" || l == "on" || l == "y") { out = 1; return true; }
  if (l == "false" || l == "no" || l == "off" || l == "n") { out = 0; return true; }
  return false;
}

bool to_int(const std::string& v, int& out) {
  char* e = nullptr;
  long x = std::strtol(v.c_str(), &e, 10);
  if (e == v.c_str() || *e != '\0') return false;
  out = (int)x;
  return true;
}

bool to_double(const std::string& v, double& out) {
  char* e = nullptr;
  double x = std::strtod(v.c_str(), &e);
  if (e == v.c_str() || *e != '\0') return false;
  out = x;
  return true;
}

}  // namespace

extern "C" LX_API lx_status lx_params_from_yaml(const char* path, lx_params* p) {
  if (!path || !p) return set_thread_error("null argument", LX_ERR_INVALID);
  std::ifstream in(path, std::ios::binary);
  if (!in) return set_thread_error((std::string("cannot open ") + path).c_str(), LX_ERR_IO);
  std::stringstream ss;
  ss << in.rdbuf();
  const std::string src = ss.str();
  Parser ps(src);
  std::vector<Doc> docs;
  for (;;) {
    Doc d;
    if (!ps.mapping(d)) break;
    docs.push_back(d);
  }
  if (!ps.err.empty()) return set_thread_error((std::string(path) + ": " + ps.err).c_str(), LX_ERR_IO);
  if (docs.size() < 5) return set_thread_error("parameters.yaml needs five documents (reader.cc:76-126)", LX_ERR_IO);

  lx_params_init(p);
  std::string bad;
  auto need = [&](int doc, const char* key) -> const std::string* {
    auto it = docs[doc].find(key);
    if (it == docs[doc].end()) {
      if (bad.empty()) bad = std::string("missing key \"") + key + "\" in document " + std::to_string(doc + 1);
      return nullptr;
    }
    return &it->second;
  };
  auto B = [&](int doc, const char* key, int& out) {
    const std::string* v = need(doc, key);
    if (v && !to_bool(*v, out) && bad.empty()) bad = std::string("\"") + key + "\" is not a boolean";
  };
  auto I = [&](int doc, const char* key, int& out) {
    const std::string* v = need(doc, key);
    if (v && !to_int(*v, out) && bad.empty()) bad = std::string("\"") + key + "\" is not an integer";
  };
  auto D = [&](int doc, const char* key, double& out) {
    const std::string* v = need(doc, key);
    if (v && !to_double(*v, out) && bad.empty()) bad = std::string("\"") + key + "\" is not a number";
  };
  B(0, "isPlanar", p->isPlanar);  // reader.cc:76-77
  I(1, "X Length", p->Nx);        // reader.cc:81-89
  I(1, "Y Length", p->Ny);
  I(1, "Z Length", p->Nz);
  D(1, "X Resolution", p->dx);
  D(1, "Y Resolution", p->dy);
  D(1, "Z Resolution", p->dz);
  D(1, "Courant factor", p->S);
  I(1, "Number of timesteps", p->num_timesteps);
  I(2, "X Number of Procs", p->npX);  // reader.cc:91-94
  I(2, "Y Number of Procs", p->npY);
  I(2, "Number of Threads per node", p->n_threads);
  B(3, "usePointSource", p->usePS);  // reader.cc:96-116
  I(3, "Source X Pos", p->Nx_source);
  I(3, "Source Y Pos", p->Ny_source);
  I(3, "Source Z Pos", p->Nz_source);
  D(3, "Source Amplitude", p->amp_source);
  D(3, "Source Omega", p->omega_source);
  B(3, "usePW", p->usePW);
  D(3, "kx_pw", p->kx_pw);
  D(3, "ky_pw", p->ky_pw);
  D(3, "kz_pw", p->kz_pw);
  D(3, "Ex_pw", p->Ex_pw);
  D(3, "Ey_pw", p->Ey_pw);
  D(3, "Ez_pw", p->Ez_pw);
  D(3, "off_pw", p->off_pw);
  I(3, "x1_pw", p->x1_pw);
  I(3, "y1_pw", p->y1_pw);
  I(3, "z1_pw", p->z1_pw);
  I(3, "x2_pw", p->x2_pw);
  I(3, "y2_pw", p->y2_pw);
  I(3, "z2_pw", p->z2_pw);
  B(4, "usePML", p->usePML);  // reader.cc:119-126
  D(4, "Thickness of PML", p->d_pml);
  D(4, "sigma_max/sigma_optimal", p->sigma);
  D(4, "m value of sigma", p->sigma_m);
  D(4, "kappa max", p->kappa);
  D(4, "max value of a", p->a_max);
  D(4, "m value for a", p->a_m);
  if (docs.size() > 5) {  // engine options, all optional
    const Doc& e = docs[5];
    auto get = [&](const char* k) -> const std::string* {
      auto it = e.find(k);
      return it == e.end() ? nullptr : &it->second;
    };
    if (auto v = get("precision")) {
      if (*v == "fp64") p->precision = LX_PREC_FP64;
      else if (*v == "fp32") p->precision = LX_PREC_FP32;
      else if (*v == "fp16") p->precision = LX_PREC_FP16S;
      else if (bad.empty()) bad = "precision must be fp64, fp32 or fp16";
    }
    if (auto v = get("pulse width")) if (!to_double(*v, p->pw_sigma) && bad.empty()) bad = "\"pulse width\" is not a number";
    if (auto v = get("cpml mode")) {
      if (*v == "reference") p->cpml_mode = LX_CPML_REFERENCE;
      else if (*v == "standard") p->cpml_mode = LX_CPML_STANDARD;
      else if (bad.empty()) bad = "cpml mode must be reference or standard";
    }
    if (auto v = get("source kind")) {
      if (*v == "cw") p->source_kind = LX_SRC_CW_HARD;
      else if (*v == "pulse") p->source_kind = LX_SRC_PULSE_SOFT;
      else if (bad.empty()) bad = "source kind must be cw or pulse";
    }
    if (auto v = get("source t0")) if (!to_double(*v, p->src_t0) && bad.empty()) bad = "\"source t0\" is not a number";
    if (auto v = get("source tw")) if (!to_double(*v, p->src_tw) && bad.empty()) bad = "\"source tw\" is not a number";
    if (auto v = get("monitor every")) if (!to_int(*v, p->monitor_every) && bad.empty()) bad = "\"monitor every\" is not an integer";
  }
  if (!bad.empty()) return set_thread_error((std::string(path) + ": " + bad).c_str(), LX_ERR_IO);
  // reader::checkData reader.cc:141-162
  if (p->npX < 1 || (p->Nx - 2) % p->npX != 0)
    return set_thread_error("ERROR: Condition-- (Number of points - 2) mod Number of processors --is not satisfied in X-direction. Aborting", LX_ERR_INVALID);
  if (p->npY < 1 || (p->Ny - 2) % p->npY != 0)
    return set_thread_error("ERROR: Condition-- (Number of points - 2) mod Number of processors --is not satisfied in Y-direction. Aborting", LX_ERR_INVALID);
  if (p->isPlanar && p->Ny != 1)
    return set_thread_error("ERROR: Please put number of grid points in Y-direction as 1 for planar solutions.", LX_ERR_INVALID);
  if (p->isPlanar && p->npY != 1)
    return set_thread_error("ERROR: Please put number of processors in Y-direction as 1 for planar solutions.", LX_ERR_INVALID);
  return LX_OK;
}
