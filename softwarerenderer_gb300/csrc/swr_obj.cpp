// Wavefront OBJ ingestion: ObjData::loadFromFile + ObjData::toVertexArray of the
// reference's examples (src/examples/ObjData.cpp:46-199), producing the vertex array
// {vertex xyz, normal xyz, texcoord uv} (8 floats per vertex, the layout of
// ObjData::VertexArrayData) and the triangle index array that VertexProcessor::drawElements
// consumes, ready for device buffers.
//
// Semantics kept from the reference:
//   * element 0 of the position, normal and texcoord lists is a zero entry, so 1-based
//     OBJ indices address the lists directly and a missing index (0, e.g. "1//3") selects
//     the zero entry;
//   * "v", "vn", "vt" read 3, 3, 2 numbers; "f" reads "v", "v/t", "v//n" or "v/t/n" words;
//     every other line, and lines whose first word starts with '#', is ignored;
//   * numbers are read as the C++ streams of the reference read them (the num_get float
//     grammar converted by strtof; leading decimal digits for indices);
//   * toVertexArray deduplicates (v, n, t) references in order of first use (std::map
//     keyed by v, then n, then t) and fans every face from its first vertex; the first
//     vertex of a face with fewer than 3 vertices is still added.
// Inputs on which the reference has undefined behaviour are rejected (SWR_EINVAL): an index
// past the end of its list (negative indices wrap past it), a word with more than three
// '/'-separated parts, an "f" line without vertices.  A "v"/"vn"/"vt" line with fewer numbers than it needs, which leaves
// the reference reading uninitialised floats, gets zeros for the missing ones.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <string>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/swr_gb300.h"

struct swr_obj_mesh {
  std::vector<float> vdata;   // 8 floats per vertex
  std::vector<int32_t> idata;
};

namespace {

struct Ref {
  uint32_t v, n, t;
  bool operator<(const Ref& o) const { return std::tie(v, n, t) < std::tie(o.v, o.n, o.t); }
};

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f'; }

// Splits a line into whitespace-separated words (istringstream >> std::string).
void split(const char* b, const char* e, std::vector<std::string>& out) {
  out.clear();
  while (b < e) {
    while (b < e && is_space(*b)) ++b;
    const char* s = b;
    while (b < e && !is_space(*b)) ++b;
    if (b > s) out.emplace_back(s, (size_t)(b - s));
  }
}

// istream >> float on the rest of a line (libstdc++ num_get): skip whitespace, take the
// longest prefix of the form [+-]digits[.digits][(e|E)[+-]digits] and convert it with
// strtof; an empty or not fully convertible prefix fails the stream (value 0), and every
// later read on a failed stream is 0 as well.  Returns the cursor after the number.
const char* read_float(const char* b, const char* e, bool& ok, float& out) {
  out = 0.0f;
  if (!ok) return b;
  while (b < e && is_space(*b)) ++b;
  const char* s = b;
  if (b < e && (*b == '+' || *b == '-')) ++b;
  while (b < e && *b >= '0' && *b <= '9') ++b;
  if (b < e && *b == '.') {
    ++b;
    while (b < e && *b >= '0' && *b <= '9') ++b;
  }
  if (b < e && (*b == 'e' || *b == 'E')) {
    ++b;
    if (b < e && (*b == '+' || *b == '-')) ++b;
    while (b < e && *b >= '0' && *b <= '9') ++b;
  }
  const std::string tok(s, (size_t)(b - s));
  char* end = nullptr;
  const float v = tok.empty() ? 0.0f : strtof(tok.c_str(), &end);
  if (tok.empty() || end != tok.c_str() + tok.size()) {
    ok = false;
    return b;
  }
  out = v;
  return b;
}

void read_floats(const char* b, const char* e, float* out, int n) {
  bool ok = true;
  for (int i = 0; i < n; ++i) b = read_float(b, e, ok, out[i]);
}

// istream >> unsigned on one part of a face word: optional sign, leading digits (the rest
// of the part is ignored); no digits -> 0; a minus sign negates modulo 2^32 and a value
// past 2^32 - 1 gives 2^32 - 1 (both then fail the list bounds check).
uint32_t parse_index(const std::string& s) {
  size_t i = 0;
  bool neg = false;
  if (i < s.size() && (s[i] == '+' || s[i] == '-')) neg = s[i++] == '-';
  uint64_t v = 0;
  bool any = false, big = false;
  for (; i < s.size() && s[i] >= '0' && s[i] <= '9'; ++i) {
    any = true;
    v = v * 10 + (uint64_t)(s[i] - '0');
    if (v > 0xffffffffull) big = true, v = 0xffffffffull + 1;
  }
  if (!any) return 0;
  if (big) return 0xffffffffu;
  return neg ? (uint32_t)(0u - (uint32_t)v) : (uint32_t)v;
}

bool parse_ref(const std::string& w, Ref& r) {
  std::string part[3];
  int k = 0;
  for (char c : w) {
    if (c == '/') {
      if (++k > 2) return false;
    } else {
      part[k] += c;
    }
  }
  // the reference reads the parts as vertex / texcoord / normal
  r.v = parse_index(part[0]);
  r.t = parse_index(part[1]);
  r.n = parse_index(part[2]);
  return true;
}

int parse(const char* text, uint64_t len, swr_obj_mesh& m) {
  std::vector<float> pos = {0, 0, 0}, nrm = {0, 0, 0}, tex = {0, 0};
  std::vector<std::vector<Ref>> faces;
  std::vector<std::string> w;
  const char* p = text;
  const char* end = text + len;
  while (p < end) {
    const char* nl = (const char*)memchr(p, '\n', (size_t)(end - p));
    const char* le = nl ? nl : end;
    const char* line = p;
    p = nl ? nl + 1 : end;
    // the command word, then the rest of the line
    const char* c = line;
    while (c < le && is_space(*c)) ++c;
    const char* ce = c;
    while (ce < le && !is_space(*ce)) ++ce;
    const std::string cmd(c, (size_t)(ce - c));
    if (cmd.empty() || cmd[0] == '#') continue;
    float f[3];
    if (cmd == "v") {
      read_floats(ce, le, f, 3);
      pos.insert(pos.end(), f, f + 3);
    } else if (cmd == "vn") {
      read_floats(ce, le, f, 3);
      nrm.insert(nrm.end(), f, f + 3);
    } else if (cmd == "vt") {
      read_floats(ce, le, f, 2);
      tex.insert(tex.end(), f, f + 2);
    } else if (cmd == "f") {
      split(ce, le, w);
      faces.emplace_back();
      for (size_t i = 0; i < w.size(); ++i) {
        Ref r;
        if (!parse_ref(w[i], r)) return SWR_EINVAL;
        faces.back().push_back(r);
      }
    }
  }
  const uint64_t np = pos.size() / 3, nn = nrm.size() / 3, nt = tex.size() / 2;
  std::map<Ref, uint32_t> seen;
  auto add = [&](const Ref& r) -> int64_t {
    auto it = seen.find(r);
    if (it != seen.end()) return it->second;
    if (r.v >= np || r.n >= nn || r.t >= nt) return -1;
    const uint32_t i = (uint32_t)seen.size();
    seen.emplace(r, i);
    m.vdata.insert(m.vdata.end(), &pos[3 * (size_t)r.v], &pos[3 * (size_t)r.v] + 3);
    m.vdata.insert(m.vdata.end(), &nrm[3 * (size_t)r.n], &nrm[3 * (size_t)r.n] + 3);
    m.vdata.insert(m.vdata.end(), &tex[2 * (size_t)r.t], &tex[2 * (size_t)r.t] + 2);
    return i;
  };
  for (const auto& f : faces) {
    if (f.empty()) return SWR_EINVAL;  // the reference reads faces[i][0] of an empty face
    const int64_t i1 = add(f[0]);
    if (i1 < 0) return SWR_EINVAL;
    for (size_t j = 2; j < f.size(); ++j) {
      const int64_t i2 = add(f[j - 1]);
      const int64_t i3 = add(f[j]);
      if (i2 < 0 || i3 < 0) return SWR_EINVAL;
      m.idata.push_back((int32_t)i1);
      m.idata.push_back((int32_t)i2);
      m.idata.push_back((int32_t)i3);
    }
    if (m.idata.size() > 0x7ffffff0u || seen.size() > 0x7ffffff0u) return SWR_EINVAL;
  }
  return SWR_OK;
}

}  // namespace

extern "C" {

int swr_obj_parse(const char* text, uint64_t len, swr_obj_mesh** out) {
  if (!out || (len && !text)) return SWR_EINVAL;
  *out = nullptr;
  swr_obj_mesh* m = new (std::nothrow) swr_obj_mesh();
  if (!m) return SWR_ENOMEM;
  const int rc = parse(text, len, *m);
  if (rc) {
    delete m;
    return rc;
  }
  *out = m;
  return SWR_OK;
}

int swr_obj_load(const char* path, swr_obj_mesh** out) {
  if (!path || !out) return SWR_EINVAL;
  *out = nullptr;
  FILE* f = fopen(path, "rb");
  if (!f) return SWR_EINVAL;
  std::string text;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
  fclose(f);
  return swr_obj_parse(text.data(), text.size(), out);
}

int swr_obj_counts(const swr_obj_mesh* m, uint64_t* nverts, uint64_t* nindices) {
  if (!m) return SWR_EINVAL;
  if (nverts) *nverts = m->vdata.size() / 8;
  if (nindices) *nindices = m->idata.size();
  return SWR_OK;
}

int swr_obj_read(const swr_obj_mesh* m, float* vdata, int32_t* idata) {
  if (!m) return SWR_EINVAL;
  if (vdata && !m->vdata.empty()) memcpy(vdata, m->vdata.data(), m->vdata.size() * sizeof(float));
  if (idata && !m->idata.empty()) memcpy(idata, m->idata.data(), m->idata.size() * sizeof(int32_t));
  return SWR_OK;
}

int swr_obj_upload(const swr_obj_mesh* m, float* vdata, int32_t* idata, void* stream) {
  if (!m) return SWR_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t vb = m->vdata.size() * sizeof(float), ib = m->idata.size() * sizeof(int32_t);
  if ((vdata && vb && cudaMemcpyAsync(vdata, m->vdata.data(), vb, cudaMemcpyHostToDevice, s) != cudaSuccess) ||
      (idata && ib && cudaMemcpyAsync(idata, m->idata.data(), ib, cudaMemcpyHostToDevice, s) != cudaSuccess) ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return SWR_ECUDA;
  }
  return SWR_OK;
}

int swr_obj_free(swr_obj_mesh* m) {
  delete m;
  return SWR_OK;
}

}  // extern "C"
