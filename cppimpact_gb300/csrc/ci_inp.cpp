// ci_inp.cpp -- Abaqus/CalculiX .inp reader behind ci_mesh_load_inp.
//
// Same accepted subset and id mapping as Mesh::load_mesh (include/mesh.h:57-267):
//  * a line starting with '*' (or empty) switches section: "*Node", "*Element",
//    "*Nset" (name after "Nset=");
//  * node lines "id, x, y, z"; element lines "id, n1, ..., n_npe" on one line;
//    node-set lines are comma lists;
//  * ids are 1-based and assumed dense: entry id-1 receives the record;
//  * slave / fixed sets are every set whose name contains "slave" / "fixed" (any
//    case), concatenated in name order (include/mesh.h:270-329).
// Unlike the reference, malformed numbers, ragged elements and ids outside the dense
// range are reported as CI_ERR_IO instead of being skipped or written out of bounds.
#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cppimpact_gb300.h"

namespace {

std::string trim(const std::string& s) {
  const char* ws = " \t\n\r\f\v";
  const size_t a = s.find_first_not_of(ws);
  if (a == std::string::npos) return "";
  const size_t b = s.find_last_not_of(ws);
  return s.substr(a, b - a + 1);
}

bool contains_icase(const std::string& s, const char* pat) {
  std::string l(s);
  std::transform(l.begin(), l.end(), l.begin(), [](unsigned char c) { return std::tolower(c); });
  return l.find(pat) != std::string::npos;
}

bool parse_double(const std::string& tok, double* v) {
  const std::string t = trim(tok);
  if (t.empty()) return false;
  char* end = nullptr;
  *v = std::strtod(t.c_str(), &end);
  return end != t.c_str();
}

bool parse_int(const std::string& tok, long* v) {
  const std::string t = trim(tok);
  if (t.empty()) return false;
  char* end = nullptr;
  *v = std::strtol(t.c_str(), &end, 10);
  return end != t.c_str();
}

}  // namespace

extern "C" int ci_mesh_load_inp(const char* path, int npe, ci_mesh* out);
extern "C" void ci_mesh_free(ci_mesh* m);

extern "C" int ci_mesh_load_inp(const char* path, int npe, ci_mesh* out) {
  if (!path || !out || (npe != 4 && npe != 10)) return CI_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  std::ifstream in(path);
  if (!in.is_open()) return CI_ERR_IO;
  std::map<long, std::vector<double>> nodes;
  std::map<long, std::vector<long>> elems;
  std::map<std::string, std::vector<long>> sets;
  enum { NONE, NODE, ELEM, NSET } sec = NONE;
  std::string cur, line;
  while (std::getline(in, line)) {
    line = trim(line);
    if (line.empty() || line[0] == '*') {
      sec = NONE;
      if (line.find("*Node") != std::string::npos) sec = NODE;
      if (line.find("*Element") != std::string::npos) sec = ELEM;
      if (line.find("*Nset") != std::string::npos) {
        sec = NSET;
        const size_t p = line.find("Nset=");
        if (p != std::string::npos) {
          cur = line.substr(p + 5);
          sets[cur];
        }
      }
      continue;
    }
    std::vector<std::string> tok;
    std::stringstream ss(line);
    std::string t;
    while (std::getline(ss, t, ',')) tok.push_back(t);
    if (sec == NODE) {
      long id;
      double x, y, z;
      if (tok.size() < 4 || !parse_int(tok[0], &id) || !parse_double(tok[1], &x) ||
          !parse_double(tok[2], &y) || !parse_double(tok[3], &z))
        return CI_ERR_IO;
      nodes[id] = {x, y, z};
    } else if (sec == ELEM) {
      std::vector<long> v;
      for (const std::string& s : tok) {
        long x;
        if (parse_int(s, &x)) v.push_back(x);
      }
      if ((int)v.size() < npe + 1) return CI_ERR_IO;
      elems[v[0]] = std::vector<long>(v.begin() + 1, v.begin() + 1 + npe);
    } else if (sec == NSET) {
      for (const std::string& s : tok) {
        long x;
        if (parse_int(s, &x)) sets[cur].push_back(x);
      }
    }
  }
  const long N = (long)nodes.size(), E = (long)elems.size();
  if (N == 0 || E == 0) return CI_ERR_IO;
  double* x = (double*)std::malloc(sizeof(double) * 3 * N);
  int* c = (int*)std::malloc(sizeof(int) * npe * E);
  if (!x || !c) {
    std::free(x);
    std::free(c);
    return CI_ERR_NOMEM;
  }
  for (const auto& kv : nodes) {
    if (kv.first < 1 || kv.first > N) {
      std::free(x);
      std::free(c);
      return CI_ERR_IO;
    }
    for (int k = 0; k < 3; k++) x[3 * (kv.first - 1) + k] = kv.second[k];
  }
  for (const auto& kv : elems) {
    if (kv.first < 1 || kv.first > E) {
      std::free(x);
      std::free(c);
      return CI_ERR_IO;
    }
    for (int a = 0; a < npe; a++) {
      const long n = kv.second[a];
      if (n < 1 || n > N) {
        std::free(x);
        std::free(c);
        return CI_ERR_IO;
      }
      c[npe * (kv.first - 1) + a] = (int)(n - 1);
    }
  }
  std::vector<int> slave, fixed;
  for (const auto& kv : sets) {
    std::vector<int>* dst = contains_icase(kv.first, "slave") ? &slave
                            : contains_icase(kv.first, "fixed") ? &fixed
                                                                : nullptr;
    if (!dst) continue;
    for (long id : kv.second) dst->push_back((int)(id - 1));
  }
  out->num_nodes = (int)N;
  out->num_elements = (int)E;
  out->nodes_per_element = npe;
  out->xloc = x;
  out->element_nodes = c;
  out->num_slave_nodes = (int)slave.size();
  out->num_fixed_nodes = (int)fixed.size();
  int* sl = (int*)std::malloc(sizeof(int) * (slave.size() + 1));
  int* fx = (int*)std::malloc(sizeof(int) * (fixed.size() + 1));
  if (!sl || !fx) {
    std::free(x);
    std::free(c);
    std::free(sl);
    std::free(fx);
    std::memset(out, 0, sizeof(*out));
    return CI_ERR_NOMEM;
  }
  std::copy(slave.begin(), slave.end(), sl);
  std::copy(fixed.begin(), fixed.end(), fx);
  out->slave_nodes = sl;
  out->fixed_nodes = fx;
  return CI_OK;
}

extern "C" void ci_mesh_free(ci_mesh* m) {
  if (!m) return;
  std::free((void*)m->xloc);
  std::free((void*)m->element_nodes);
  std::free((void*)m->slave_nodes);
  std::free((void*)m->fixed_nodes);
  std::memset(m, 0, sizeof(*m));
}
