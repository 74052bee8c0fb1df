// gpv_mesh.cpp -- host side: .obj/.off loaders with the reference's semantics, the .raw writer
// and reader (the synthetic mesh generators are in gpv_meshgen.cpp).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/gpview.h"

namespace {

// ---- loaders -----------------------------------------------------------------------------------

// Splits on one separator the way the reference's split() does (src/Utilities.cpp:989-1005):
// consecutive separators give empty words and a trailing separator gives one trailing empty word.
std::vector<std::string> split_on(const std::string &s, const std::string &tok) {
  std::vector<std::string> out;
  std::string str = s;
  while (!str.empty()) {
    size_t idx = str.find(tok);
    if (idx != std::string::npos) {
      out.push_back(str.substr(0, idx));
      str = str.substr(idx + tok.size());
      if (str.empty()) out.push_back(str);
    } else {
      out.push_back(str);
      str.clear();
    }
  }
  return out;
}

bool parse_float(const std::string &w, float &v) {
  if (w.empty()) return false;
  char *end = nullptr;
  v = std::strtof(w.c_str(), &end);
  return end != w.c_str();
}

bool parse_int(const std::string &w, int &v) {
  if (w.empty()) return false;
  char *end = nullptr;
  long x = std::strtol(w.c_str(), &end, 10);
  if (end == w.c_str()) return false;
  v = (int)x;
  return true;
}

float magnitude(const float a[3]) {
  // VectorMagnitude (includes/FloatVector.h:323-326): float products and sum, sqrt.
  float s = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  return (float)std::sqrt((double)s);
}

// Padding and model size shared by both loaders (src/Object.cpp:572-583, :285-296).
void finish_bounds(float mn[3], float mx[3], gpv_mesh *m) {
  float d[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
  double model_size = magnitude(d);
  float offset = (float)(0.001 * model_size);
  for (int a = 0; a < 3; ++a) {
    m->bbox_max[a] = offset + mx[a];
    m->bbox_min[a] = mn[a] - offset;
  }
  float ex = m->bbox_max[0] - m->bbox_min[0], ey = m->bbox_max[1] - m->bbox_min[1],
        ez = m->bbox_max[2] - m->bbox_min[2];
  m->max_model_size = ex > (ey > ez ? ey : ez) ? ex : (ey > ez ? ey : ez);
}

int store(const std::vector<float> &v, gpv_mesh *m) {
  m->num_triangles = (int64_t)(v.size() / 9);
  m->tris = (float *)std::malloc(sizeof(float) * (v.size() ? v.size() : 1));
  if (!m->tris) return GPV_ERR_OOM;
  if (!v.empty()) std::memcpy(m->tris, v.data(), sizeof(float) * v.size());
  return GPV_OK;
}

}  // namespace

extern "C" {

int gpv_load_obj(const char *path, gpv_mesh *out) {
  if (!path || !out) return GPV_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  std::ifstream in(path, std::ios::in);
  if (!in.good()) return GPV_ERR_IO;
  std::vector<float> verts;
  std::vector<float> tris;
  float mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
  int64_t nv = 0;
  // Like Object::ReadObject (src/Object.cpp:395-584): a line is processed only while the stream
  // is still good after reading it, so an unterminated last line is ignored.
  while (in.good()) {
    std::string line;
    std::getline(in, line);
    std::vector<std::string> w1 = split_on(line, " "), w2 = split_on(line, "\t");
    const std::vector<std::string> &w = w1.size() > w2.size() ? w1 : w2;
    if (!in.good()) break;
    if (w.empty() || w[0].empty()) continue;
    if (w[0][0] == 'v' && w[0].size() == 1) {
      if (w.size() < 4) return GPV_ERR_PARSE;
      float p[3];
      for (int i = 0; i < 3; ++i)
        if (!parse_float(w[1 + i], p[i])) return GPV_ERR_PARSE;
      for (int a = 0; a < 3; ++a) {
        if (nv == 0) { mn[a] = p[a]; mx[a] = p[a]; }
        else {
          mn[a] = mn[a] < p[a] ? mn[a] : p[a];
          mx[a] = mx[a] > p[a] ? mx[a] : p[a];
        }
        verts.push_back(p[a]);
      }
      ++nv;
    } else if (w[0][0] == 'f' && w[0].size() == 1) {
      if (w.size() != 4) return GPV_ERR_PARSE;  // the reference asserts exactly 3 vertices
      int idx[3];
      for (int i = 0; i < 3; ++i) {
        std::vector<std::string> parts = split_on(w[1 + i], "/");
        const std::string &first = parts.size() <= 1 ? w[1 + i] : parts[0];
        if (!parse_int(first, idx[i])) return GPV_ERR_PARSE;
        idx[i] -= 1;
        if (idx[i] < 0 || idx[i] >= nv) return GPV_ERR_PARSE;
      }
      for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 3; ++a) tris.push_back(verts[3 * (size_t)idx[i] + a]);
    }
  }
  if (nv == 0) return GPV_ERR_PARSE;
  finish_bounds(mn, mx, out);
  return store(tris, out);
}

int gpv_load_off(const char *path, gpv_mesh *out) {
  if (!path || !out) return GPV_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  std::ifstream in(path, std::ios::in);
  if (!in.good()) return GPV_ERR_IO;
  std::string header;
  long nv = 0, nf = 0, ne = 0;
  if (!(in >> header >> nv >> nf >> ne) || nv <= 0 || nf < 0) return GPV_ERR_PARSE;
  std::vector<float> verts((size_t)nv * 3);
  for (long i = 0; i < nv; ++i)
    if (!(in >> verts[3 * i] >> verts[3 * i + 1] >> verts[3 * i + 2])) return GPV_ERR_PARSE;
  std::vector<float> tris;
  tris.reserve((size_t)nf * 9);
  for (long f = 0; f < nf; ++f) {
    long cnt;
    long idx[3];
    if (!(in >> cnt >> idx[0] >> idx[1] >> idx[2]) || cnt < 3) return GPV_ERR_PARSE;
    // Object::ReadOFFObject uses the first three indices of a face (src/Object.cpp:215-249);
    // extra indices of larger polygons are skipped here.
    for (long e = 3; e < cnt; ++e) {
      long skip;
      if (!(in >> skip)) return GPV_ERR_PARSE;
    }
    for (int i = 0; i < 3; ++i) {
      if (idx[i] < 0 || idx[i] >= nv) return GPV_ERR_PARSE;
      for (int a = 0; a < 3; ++a) tris.push_back(verts[3 * idx[i] + a]);
    }
  }
  if (nf == 0) return GPV_ERR_PARSE;
  // bounds over the triangles' vertices (src/Object.cpp:262-271)
  float mn[3], mx[3];
  for (int a = 0; a < 3; ++a) mn[a] = mx[a] = tris[a];
  for (size_t k = 0; k < tris.size(); k += 3)
    for (int a = 0; a < 3; ++a) {
      float p = tris[k + a];
      mn[a] = mn[a] < p ? mn[a] : p;
      mx[a] = mx[a] > p ? mx[a] : p;
    }
  finish_bounds(mn, mx, out);
  return store(tris, out);
}

void gpv_mesh_free(gpv_mesh *mesh) {
  if (!mesh) return;
  std::free(mesh->tris);
  mesh->tris = nullptr;
  mesh->num_triangles = 0;
}

int gpv_write_raw(const char *prefix, const gpv_result *res, const uint8_t *level1_inout,
                  const int32_t *level1_prefix, const uint8_t *level2_inout) {
  if (!prefix || !res || !level1_inout) return GPV_ERR_INVALID;
  const std::string p(prefix);
  const gpv_grid_spec &s = res->spec;
  const bool l2 = s.ndiv2[0] > 0;
  {
    // VoxelConfig.txt (src/Object.cpp:3009-3022), default stream formatting
    std::ofstream cfg(p + "VoxelConfig.txt");
    if (!cfg.good()) return GPV_ERR_IO;
    cfg << p << "\n";
    cfg << s.bbox_min[0] << "\t" << s.bbox_min[1] << "\t" << s.bbox_min[2] << "\n";
    cfg << s.bbox_max[0] << "\t" << s.bbox_max[1] << "\t" << s.bbox_max[2] << "\n";
    cfg << s.ndiv[0] << "\t" << s.ndiv[1] << "\t" << s.ndiv[2] << "\n";
    cfg << res->grid_size[0] << "\t" << res->grid_size[1] << "\t" << res->grid_size[2] << "\n";
    cfg << res->num_level1_inside << "\n" << res->num_boundary << "\n";
    if (l2) {
      cfg << s.ndiv2[0] << "\t" << s.ndiv2[1] << "\t" << s.ndiv2[2] << "\n";
      cfg << res->grid_size2[0] << "\t" << res->grid_size2[1] << "\t" << res->grid_size2[2] << "\n";
      cfg << res->num_level2_inside << "\n" << res->num_level2_boundary << "\n";
    }
    if (!cfg.good()) return GPV_ERR_IO;
  }
  auto dump = [&](const std::string &name, const void *data, size_t bytes) -> int {
    std::ofstream f(p + name, std::ios::binary);
    if (!f.good()) return GPV_ERR_IO;
    if (bytes) f.write((const char *)data, (std::streamsize)bytes);
    return f.good() ? GPV_OK : GPV_ERR_IO;
  };
  int rc = dump("Level1InOut.raw", level1_inout, (size_t)res->num_level1);
  if (rc) return rc;
  if (l2) {
    if (!level1_prefix || (res->num_boundary && !level2_inout)) return GPV_ERR_INVALID;
    rc = dump("Level1BoundaryPrefixSum.raw", level1_prefix, sizeof(int32_t) * (size_t)res->num_level1);
    if (rc) return rc;
    const size_t cells = (size_t)s.ndiv2[0] * s.ndiv2[1] * s.ndiv2[2];
    rc = dump("Level2InOut.raw", level2_inout, (size_t)res->num_boundary * cells);
    if (rc) return rc;
  }
  return GPV_OK;
}

int gpv_write_raw_normals(const char *prefix, const gpv_result *res, const uint8_t *level1_normal,
                          const uint8_t *level2_normal) {
  if (!prefix || !res || !level1_normal) return GPV_ERR_INVALID;
  const std::string p(prefix);
  const gpv_grid_spec &s = res->spec;
  const bool l2 = s.ndiv2[0] > 0;
  if (l2 && res->num_boundary && !level2_normal) return GPV_ERR_INVALID;
  auto dump = [&](const std::string &name, const void *data, size_t bytes) -> int {
    std::ofstream f(p + name, std::ios::binary);
    if (!f.good()) return GPV_ERR_IO;
    if (bytes) f.write((const char *)data, (std::streamsize)bytes);
    return f.good() ? GPV_OK : GPV_ERR_IO;
  };
  int rc = dump("Level1Normal.raw", level1_normal, 3 * (size_t)res->num_level1);
  if (rc || !l2) return rc;
  const size_t cells = (size_t)s.ndiv2[0] * s.ndiv2[1] * s.ndiv2[2];
  return dump("Level2Normal.raw", level2_normal, 3 * (size_t)res->num_boundary * cells);
}

int gpv_read_voxel_config(const char *prefix, gpv_voxel_config *out) {
  if (!prefix || !out) return GPV_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  std::ifstream f(std::string(prefix) + "VoxelConfig.txt");
  if (!f.good()) return GPV_ERR_IO;
  std::string name;
  if (!std::getline(f, name)) return GPV_ERR_PARSE;
  auto rd3f = [&](float *v) { return static_cast<bool>(f >> v[0] >> v[1] >> v[2]); };
  auto rd3i = [&](int32_t *v) { return static_cast<bool>(f >> v[0] >> v[1] >> v[2]); };
  long long a = 0, b = 0;
  if (!rd3f(out->bbox_min) || !rd3f(out->bbox_max) || !rd3i(out->ndiv) || !rd3f(out->grid_size) ||
      !(f >> a >> b))
    return GPV_ERR_PARSE;
  out->num_level1_inside = a;
  out->num_boundary = b;
  for (int k = 0; k < 3; ++k)
    if (out->ndiv[k] < 1) return GPV_ERR_PARSE;
  int32_t n2[3];
  if (rd3i(n2)) {  // the Level2 block is present
    float g2[3];
    if (!rd3f(g2) || !(f >> a >> b)) return GPV_ERR_PARSE;
    for (int k = 0; k < 3; ++k) {
      if (n2[k] < 1) return GPV_ERR_PARSE;
      out->ndiv2[k] = n2[k];
      out->grid_size2[k] = g2[k];
    }
    out->has_level2 = 1;
    out->num_level2_inside = a;
    out->num_level2_boundary = b;
  }
  return GPV_OK;
}

int gpv_read_raw(const char *prefix, const gpv_voxel_config *cfg, uint8_t *level1_inout,
                 int32_t *level1_prefix, uint8_t *level2_inout, uint8_t *level1_normal,
                 uint8_t *level2_normal) {
  if (!prefix || !cfg) return GPV_ERR_INVALID;
  const std::string p(prefix);
  const size_t N1 = (size_t)cfg->ndiv[0] * cfg->ndiv[1] * cfg->ndiv[2];
  const size_t cells = cfg->has_level2 ? (size_t)cfg->ndiv2[0] * cfg->ndiv2[1] * cfg->ndiv2[2] : 0;
  const size_t L2 = (size_t)cfg->num_boundary * cells;
  if ((level1_prefix || level2_inout || level2_normal) && !cfg->has_level2) return GPV_ERR_INVALID;
  auto load = [&](const char *name, void *dst, size_t bytes) -> int {
    if (!dst) return GPV_OK;
    std::ifstream f(p + name, std::ios::binary);
    if (!f.good()) return GPV_ERR_IO;
    if (bytes) f.read(static_cast<char *>(dst), (std::streamsize)bytes);
    return (size_t)f.gcount() == bytes ? GPV_OK : GPV_ERR_IO;
  };
  int rc = load("Level1InOut.raw", level1_inout, N1);
  if (!rc) rc = load("Level1BoundaryPrefixSum.raw", level1_prefix, 4 * N1);
  if (!rc) rc = load("Level2InOut.raw", level2_inout, L2);
  if (!rc) rc = load("Level1Normal.raw", level1_normal, 3 * N1);
  if (!rc) rc = load("Level2Normal.raw", level2_normal, 3 * L2);
  return rc;
}

}  // extern "C"
