// mesh_io.cpp - host-side mesh reading, edge extraction and ground-truth
// comparison (include/stq_io.h). No third-party parsers: small readers for
// the subset of OBJ, PLY and JSON that the reference's inputs use.
#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "../../include/stq_io.h"

namespace {

struct MeshData {
  std::vector<double> V;
  std::vector<int32_t> F;
};

bool ends_with(const std::string &s, const char *suffix) {
  const size_t n = std::strlen(suffix);
  if (s.size() < n) return false;
  for (size_t i = 0; i < n; ++i)
    if (std::tolower(static_cast<unsigned char>(s[s.size() - n + i])) != suffix[i]) return false;
  return true;
}

// OBJ: "v x y z [w]" and "f i[/t[/n]] j... k..." (1-based; negative = relative).
bool read_obj(const std::string &path, MeshData &m) {
  std::ifstream in(path);
  if (!in) return false;
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ss(line);
    std::string tag;
    if (!(ss >> tag)) continue;
    if (tag == "v") {
      double x, y, z;
      if (!(ss >> x >> y >> z)) return false;
      m.V.push_back(x), m.V.push_back(y), m.V.push_back(z);
    } else if (tag == "f") {
      std::string tok;
      int32_t idx[3];
      int k = 0;
      while (ss >> tok) {
        if (k == 3) return false;  // only triangles
        const long v = std::strtol(tok.c_str(), nullptr, 10);
        const long nv = long(m.V.size() / 3);
        const long i = v > 0 ? v - 1 : nv + v;
        if (v == 0 || i < 0) return false;
        idx[k++] = int32_t(i);
      }
      if (k != 3) return false;
      m.F.insert(m.F.end(), idx, idx + 3);
    }
  }
  return true;
}

// PLY: header, then vertex and face elements (ascii or binary little endian).
bool read_ply(const std::string &path, MeshData &m) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return false;
  std::string line;
  if (!std::getline(in, line) || line.rfind("ply", 0) != 0) return false;
  bool binary = false;
  struct Elem {
    std::string name;
    int64_t count = 0;
    std::vector<std::pair<std::string, std::string>> props;  // (type, name); list: ("list cnt item", name)
  };
  std::vector<Elem> elems;
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    std::istringstream ss(line);
    std::string w;
    ss >> w;
    if (w == "format") {
      std::string f;
      ss >> f;
      if (f == "binary_little_endian") binary = true;
      else if (f != "ascii") return false;
    } else if (w == "element") {
      Elem e;
      ss >> e.name >> e.count;
      elems.push_back(e);
    } else if (w == "property") {
      if (elems.empty()) return false;
      std::string t;
      ss >> t;
      if (t == "list") {
        std::string ct, it, name;
        ss >> ct >> it >> name;
        elems.back().props.push_back({"list " + ct + " " + it, name});
      } else {
        std::string name;
        ss >> name;
        elems.back().props.push_back({t, name});
      }
    } else if (w == "end_header") {
      break;
    }
  }
  auto size_of = [](const std::string &t) -> int {
    if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
    if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
    if (t == "int" || t == "uint" || t == "float" || t == "int32" || t == "uint32" || t == "float32") return 4;
    if (t == "double" || t == "float64") return 8;
    return 0;
  };
  auto read_bin = [&](const std::string &t, double &out) -> bool {
    unsigned char buf[8];
    const int n = size_of(t);
    if (!n || !in.read(reinterpret_cast<char *>(buf), n)) return false;
    if (t == "char" || t == "int8") out = double(int8_t(buf[0]));
    else if (t == "uchar" || t == "uint8") out = double(buf[0]);
    else if (t == "short" || t == "int16") { int16_t v; std::memcpy(&v, buf, 2); out = v; }
    else if (t == "ushort" || t == "uint16") { uint16_t v; std::memcpy(&v, buf, 2); out = v; }
    else if (t == "int" || t == "int32") { int32_t v; std::memcpy(&v, buf, 4); out = v; }
    else if (t == "uint" || t == "uint32") { uint32_t v; std::memcpy(&v, buf, 4); out = v; }
    else if (t == "float" || t == "float32") { float v; std::memcpy(&v, buf, 4); out = v; }
    else { double v; std::memcpy(&v, buf, 8); out = v; }
    return true;
  };
  for (const Elem &e : elems) {
    const bool is_v = e.name == "vertex", is_f = e.name == "face";
    for (int64_t r = 0; r < e.count; ++r) {
      double xyz[3] = {0, 0, 0};
      std::vector<int64_t> list;
      std::istringstream row;
      if (!binary) {
        if (!std::getline(in, line)) return false;
        row.str(line);
      }
      for (const auto &pr : e.props) {
        if (pr.first.rfind("list", 0) == 0) {
          std::istringstream lt(pr.first);
          std::string l, ct, it;
          lt >> l >> ct >> it;
          double cnt = 0;
          if (binary ? !read_bin(ct, cnt) : !(row >> cnt)) return false;
          for (int64_t q = 0; q < int64_t(cnt); ++q) {
            double v = 0;
            if (binary ? !read_bin(it, v) : !(row >> v)) return false;
            list.push_back(int64_t(v));
          }
        } else {
          double v = 0;
          if (binary ? !read_bin(pr.first, v) : !(row >> v)) return false;
          if (pr.second == "x") xyz[0] = v;
          else if (pr.second == "y") xyz[1] = v;
          else if (pr.second == "z") xyz[2] = v;
        }
      }
      if (is_v) m.V.insert(m.V.end(), xyz, xyz + 3);
      if (is_f) {
        if (list.size() != 3) return false;
        for (int64_t v : list) m.F.push_back(int32_t(v));
      }
    }
  }
  return true;
}

}  // namespace

extern "C" {

int stq_read_mesh(const char *path, double *V, int64_t *nV, int32_t *F, int64_t *nF) {
  if (!path || !nV || !nF) return STQ_ERR_INVALID_ARG;
  MeshData m;
  const std::string p(path);
  const bool ok = ends_with(p, ".obj") ? read_obj(p, m) : ends_with(p, ".ply") ? read_ply(p, m) : false;
  if (!ok) return STQ_ERR_INVALID_INPUT;
  const int64_t nv = int64_t(m.V.size() / 3), nf = int64_t(m.F.size() / 3);
  for (int32_t i : m.F)
    if (i < 0 || i >= nv) return STQ_ERR_INVALID_INPUT;
  if (V || F) {
    if (!V || !F || *nV < nv || *nF < nf) return STQ_ERR_INVALID_ARG;
    std::copy(m.V.begin(), m.V.end(), V);
    std::copy(m.F.begin(), m.F.end(), F);
  }
  *nV = nv;
  *nF = nf;
  return STQ_OK;
}

int stq_mesh_edges(const int32_t *F, int64_t nF, int32_t *E, int64_t *nE) {
  if (!nE || nF < 0 || (nF > 0 && !F)) return STQ_ERR_INVALID_ARG;
  std::vector<uint64_t> keys;
  keys.reserve(size_t(3 * nF));
  for (int64_t f = 0; f < nF; ++f)
    for (int k = 0; k < 3; ++k) {
      const uint32_t a = uint32_t(F[3 * f + k]), b = uint32_t(F[3 * f + (k + 1) % 3]);
      if (a == b) continue;
      const uint32_t lo = std::min(a, b), hi = std::max(a, b);
      keys.push_back((uint64_t(hi) << 32) | lo);  // order by (larger, smaller)
    }
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  if (E) {
    if (*nE < int64_t(keys.size())) return STQ_ERR_INVALID_ARG;
    for (size_t k = 0; k < keys.size(); ++k) {
      E[2 * k] = int32_t(keys[k] & 0xffffffffu);
      E[2 * k + 1] = int32_t(keys[k] >> 32);
    }
  }
  *nE = int64_t(keys.size());
  return STQ_OK;
}

int stq_compare_truth_json(const char *path, const stq_pair *h_pairs, int64_t count, int64_t *found,
                           int64_t *truth, int64_t *extra) {
  if (!path || !found || !truth || count < 0 || (count > 0 && !h_pairs)) return STQ_ERR_INVALID_ARG;
  std::ifstream in(path);
  if (!in) return STQ_ERR_INVALID_INPUT;
  const std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  // [[a, b], [c, d], ...]: integers at nesting depth 2, two per inner array
  std::vector<uint64_t> t;
  int depth = 0, k = 0;
  long long cur[2] = {0, 0};
  for (size_t i = 0; i < text.size();) {
    const char c = text[i];
    if (c == '[') {
      ++depth, ++i;
      if (depth == 2) k = 0;
    } else if (c == ']') {
      if (depth == 2) {
        if (k != 2) return STQ_ERR_INVALID_INPUT;
        const uint64_t lo = uint64_t(std::min(cur[0], cur[1])), hi = uint64_t(std::max(cur[0], cur[1]));
        t.push_back((lo << 32) | hi);
      }
      --depth, ++i;
    } else if (c == '-' || std::isdigit(static_cast<unsigned char>(c))) {
      char *endp = nullptr;
      const long long v = std::strtoll(text.c_str() + i, &endp, 10);
      if (depth != 2 || k >= 2 || v < 0 || v > INT32_MAX) return STQ_ERR_INVALID_INPUT;
      cur[k++] = v;
      i = size_t(endp - text.c_str());
    } else {
      ++i;
    }
  }
  if (depth != 0) return STQ_ERR_INVALID_INPUT;
  std::sort(t.begin(), t.end());
  t.erase(std::unique(t.begin(), t.end()), t.end());
  std::vector<uint64_t> a(static_cast<size_t>(count));
  for (int64_t q = 0; q < count; ++q) {
    const uint32_t x = uint32_t(h_pairs[q].first), y = uint32_t(h_pairs[q].second);
    a[size_t(q)] = (uint64_t(std::min(x, y)) << 32) | std::max(x, y);
  }
  std::sort(a.begin(), a.end());
  a.erase(std::unique(a.begin(), a.end()), a.end());
  int64_t both = 0;
  size_t i = 0, j = 0;
  while (i < t.size() && j < a.size()) {
    if (t[i] == a[j]) ++both, ++i, ++j;
    else if (t[i] < a[j]) ++i;
    else ++j;
  }
  *found = both;
  *truth = int64_t(t.size());
  if (extra) *extra = int64_t(a.size()) - both;
  return STQ_OK;
}

}  // extern "C"
