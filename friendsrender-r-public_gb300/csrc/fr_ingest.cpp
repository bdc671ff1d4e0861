// Scene ingest: Scene::CreateScene (Scene.cpp:13-218) on the host.
//
// The OBJ and MTL text is read the way tinyobjloader 0.9.22 (the version the
// reference vendors as tiny_obj_loader.cpp) reads it with its default flags
// (triangulation on, normal generation off), restated here from its behaviour:
//  * lines end at '\n', "\r\n" or '\r'; leading blanks are skipped; '#'
//    starts a comment line;
//  * numbers are parsed by its own decimal parser (tiny_obj_loader.cpp:
//    140-250: the integer digits accumulated as m = m * 10 + d, each fraction
//    digit added as d * 10^-k, the result m * 5^e scaled by 2^e), not strtod;
//  * a face "f" holds i, i/j, i//k or i/j/k triples (1-based, negative =
//    relative to the end); polygons become fans (v0, v[k-1], v[k]);
//  * faces collect in a face group that is flushed into the current shape on
//    "usemtl" (when the material changes), "g", "o" and at the end; the shape
//    is kept at "g", "o" and the end only when that last flush had faces
//    (tiny_obj_loader.cpp:887-990,1052-1056), so faces flushed by a usemtl
//    right before a "g" or "o" are dropped, as in the reference;
//  * a flush de-duplicates (v, vt, vn) triples within the group; a vertex
//    appends its normal / texcoord to the shape's arrays only when it has a
//    valid one, and the shape's facets index those arrays by vertex number
//    (Scene.cpp:93-140);
//  * "mtllib" loads asset_dir + name; a file that cannot be read still adds
//    one default material named "" (the loader's final flush).
// The facets then follow Scene.cpp:60-208: per shape, per triangle: the
// three positions, the shape's normals (or, when the shape has none, the face
// normal (p1 - p2)^ x (p2 - p0)^ of Vec3::normalized, Vec.h:240-243), the
// texcoords (or 0), and the face's material.  Reads that the reference makes
// past the end of a shape's normal or texcoord array (undefined there) are
// errors here.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/friendsrender.h"
#include "fr_ingest.h"

struct fr_scene {
  fr_scene_desc desc{};
  std::vector<float> positions, normals, uvs;
  std::vector<int32_t> material_ids;
  std::vector<fr_material_desc> materials;
  std::vector<std::string> material_names;
  std::vector<std::vector<uint8_t>> texels;
  std::vector<fr_texture_desc> textures;
  std::vector<uint8_t> env_texels;
  fr_texture_desc environment{};
};

namespace fr {
namespace {

bool is_blank(char c) { return c == ' ' || c == '\t'; }
bool is_line_end(char c) { return c == '\r' || c == '\n' || c == '\0'; }
bool is_digit(char c) { return (unsigned)(c - '0') < 10u; }

// Calls fn(line) for each line of text, lines ending at "\n", "\r\n" or
// "\r" (a last line without an ending counts when it is not empty).
template <class Fn>
void for_each_line(const std::string& text, Fn fn) {
  std::string cur;
  size_t i = 0;
  const size_t n = text.size();
  while (i < n) {
    size_t j = i;
    while (j < n && text[j] != '\n' && text[j] != '\r') ++j;
    cur.assign(text, i, j - i);
    if (j < n) {
      if (text[j] == '\r' && j + 1 < n && text[j + 1] == '\n') ++j;
      fn(cur);
    } else if (!cur.empty()) {
      fn(cur);
    }
    i = j + 1;
  }
}

bool read_file(const std::string& path, std::string* text) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t got;
  text->clear();
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text->append(buf, got);
  std::fclose(f);
  return true;
}

// 10^-k for the fraction digits, from the same pow the loader calls.
double pow10_neg(int k) {
  static const struct Table {
    double v[40];
    Table() {
      for (int i = 0; i < 40; ++i) v[i] = std::pow(10.0, -i);
    }
  } table;
  return k < 40 ? table.v[k] : std::pow(10.0, -k);
}

// The loader's decimal parser over [s, end); false (value untouched) when the
// text is not a number.
bool parse_decimal(const char* s, const char* end, double* result) {
  if (s >= end) return false;
  double mantissa = 0.0;
  int exponent = 0;
  int sign = 1, exp_sign = 1;
  const char* c = s;
  if (*c == '+' || *c == '-') {
    sign = *c == '-' ? -1 : 1;
    ++c;
  } else if (!is_digit(*c)) {
    return false;
  }
  int read = 0;
  while (c != end && is_digit(*c)) {
    mantissa *= 10;
    mantissa += (int)(*c - '0');
    ++c;
    ++read;
  }
  if (read == 0) return false;
  if (c != end) {
    if (*c == '.') {
      ++c;
      read = 1;
      while (c != end && is_digit(*c)) {
        mantissa += (int)(*c - '0') * pow10_neg(read);
        ++read;
        ++c;
      }
    } else if (*c != 'e' && *c != 'E') {
      goto assemble;
    }
    if (c != end && (*c == 'e' || *c == 'E')) {
      ++c;
      if (c != end && (*c == '+' || *c == '-')) {
        exp_sign = *c == '-' ? -1 : 1;
        ++c;
      } else if (!is_digit(*c)) {
        return false;
      }
      read = 0;
      while (c != end && is_digit(*c)) {
        exponent *= 10;
        exponent += (int)(*c - '0');
        ++c;
        ++read;
      }
      exponent *= exp_sign;
      if (read == 0) return false;
    }
  }
assemble:
  *result = sign * std::ldexp(mantissa * std::pow(5.0, exponent), exponent);
  return true;
}

// One number: skip blanks, parse up to the next blank or '\r'; 0 when it is
// not a number.
float parse_float(const char*& t) {
  t += std::strspn(t, " \t");
  const char* end = t + std::strcspn(t, " \t\r");
  double v = 0.0;
  parse_decimal(t, end, &v);
  t = end;
  return (float)v;
}

// atoi: optional blanks and sign, then digits.
int parse_int(const char* t) {
  while (*t == ' ' || *t == '\t' || *t == '\n' || *t == '\v' || *t == '\f' || *t == '\r') ++t;
  long long v = 0;
  int sign = 1;
  if (*t == '+' || *t == '-') sign = *t++ == '-' ? -1 : 1;
  while (is_digit(*t) && v < (1ll << 40)) v = v * 10 + (*t++ - '0');
  v *= sign;
  if (v > 0x7FFFFFFF) v = 0x7FFFFFFF;
  if (v < -0x7FFFFFFFll - 1) v = -0x7FFFFFFFll - 1;
  return (int)v;
}

// sscanf("%s"): the first run of non-space characters ("" when none).
std::string first_word(const char* t) {
  while (*t && std::strchr(" \t\r\n\v\f", *t)) ++t;
  const char* e = t;
  while (*e && !std::strchr(" \t\r\n\v\f", *e)) ++e;
  return std::string(t, e);
}

int fix_index(int idx, int n) { return idx > 0 ? idx - 1 : idx == 0 ? 0 : n + idx; }

struct VertexRef {
  int v, vt, vn;
  bool operator==(const VertexRef& o) const { return v == o.v && vt == o.vt && vn == o.vn; }
};
struct VertexRefHash {
  size_t operator()(const VertexRef& r) const {
    uint64_t h = (uint64_t)(uint32_t)r.v * 0x9E3779B97F4A7C15ull;
    h ^= (uint64_t)(uint32_t)r.vt * 0xC2B2AE3D27D4EB4Full + (h >> 29);
    h ^= (uint64_t)(uint32_t)r.vn * 0x165667B19E3779F9ull + (h >> 31);
    return (size_t)h;
  }
};

VertexRef parse_triple(const char*& t, int nv, int nvn, int nvt) {
  VertexRef r{-1, -1, -1};
  r.v = fix_index(parse_int(t), nv);
  t += std::strcspn(t, "/ \t\r");
  if (t[0] != '/') return r;
  ++t;
  if (t[0] == '/') {  // i//k
    ++t;
    r.vn = fix_index(parse_int(t), nvn);
    t += std::strcspn(t, "/ \t\r");
    return r;
  }
  r.vt = fix_index(parse_int(t), nvt);  // i/j or i/j/k
  t += std::strcspn(t, "/ \t\r");
  if (t[0] != '/') return r;
  ++t;
  r.vn = fix_index(parse_int(t), nvn);
  t += std::strcspn(t, "/ \t\r");
  return r;
}

struct Shape {
  std::vector<float> positions, normals, texcoords;
  std::vector<uint32_t> indices;
  std::vector<int32_t> material_ids;  // one per triangle
};

struct MtlMaterial {
  std::string name;
  float kd[3] = {0, 0, 0}, ke[3] = {0, 0, 0};
  std::string map_kd, map_d, map_bump;  // map_Ks is read by the reference's loader but never used
};

struct ObjData {
  std::vector<float> v, vn, vt;
  std::vector<Shape> shapes;
  std::vector<MtlMaterial> materials;
  std::map<std::string, int> material_map;
};

// LoadMtl (tiny_obj_loader.cpp:505-728), the keys CreateScene reads.
void load_mtl(const std::string& path, ObjData* obj) {
  std::string text;
  const bool ok = read_file(path, &text);
  MtlMaterial m;
  auto flush = [&](const MtlMaterial& mat) {
    obj->material_map.insert({mat.name, (int)obj->materials.size()});
    obj->materials.push_back(mat);
  };
  if (ok) {
    for_each_line(text, [&](const std::string& line) {
      const char* t = line.c_str();
      t += std::strspn(t, " \t");
      if (t[0] == '\0' || t[0] == '#') return;
      if (!std::strncmp(t, "newmtl", 6) && is_blank(t[6])) {
        if (!m.name.empty()) flush(m);
        m = MtlMaterial();
        m.name = first_word(t + 7);
        return;
      }
      if (t[0] == 'K' && t[1] == 'd' && is_blank(t[2])) {
        t += 2;
        for (float& x : m.kd) x = parse_float(t);
        return;
      }
      if (t[0] == 'K' && t[1] == 'e' && is_blank(t[2])) {
        t += 2;
        for (float& x : m.ke) x = parse_float(t);
        return;
      }
      if (!std::strncmp(t, "map_Kd", 6) && is_blank(t[6])) {
        m.map_kd = t + 7;
        return;
      }
      if (!std::strncmp(t, "map_bump", 8) && is_blank(t[8])) {
        m.map_bump = t + 9;
        return;
      }
      if (!std::strncmp(t, "map_d", 5) && is_blank(t[5])) {
        m.map_d = t + 6;
        return;
      }
      if (!std::strncmp(t, "bump", 4) && is_blank(t[4])) {
        m.map_bump = t + 5;
        return;
      }
    });
  }
  flush(m);  // the last material, or a default one named "" (also for a file that cannot be read)
}

// exportFaceGroupToShape (tiny_obj_loader.cpp:401-500) with triangulation:
// false when the group is empty.
bool flush_group(const ObjData& obj, const std::vector<std::vector<VertexRef>>& group, int material, Shape* shape,
                 std::string* error) {
  if (group.empty()) return false;
  std::unordered_map<VertexRef, uint32_t, VertexRefHash> cache;
  auto vertex = [&](const VertexRef& r, uint32_t* idx) -> bool {
    auto it = cache.find(r);
    if (it != cache.end()) {
      *idx = it->second;
      return true;
    }
    if (r.v < 0 || (size_t)r.v * 3 + 2 >= obj.v.size()) {
      *error = "face refers to vertex " + std::to_string(r.v + 1) + " of " + std::to_string(obj.v.size() / 3);
      return false;
    }
    for (int k = 0; k < 3; ++k) shape->positions.push_back(obj.v[(size_t)r.v * 3 + k]);
    if (r.vn >= 0 && (size_t)r.vn * 3 + 2 < obj.vn.size())
      for (int k = 0; k < 3; ++k) shape->normals.push_back(obj.vn[(size_t)r.vn * 3 + k]);
    if (r.vt >= 0 && (size_t)r.vt * 2 + 1 < obj.vt.size())
      for (int k = 0; k < 2; ++k) shape->texcoords.push_back(obj.vt[(size_t)r.vt * 2 + k]);
    *idx = (uint32_t)(shape->positions.size() / 3 - 1);
    cache.emplace(r, *idx);
    return true;
  };
  for (const auto& face : group) {
    if (face.size() < 3) continue;  // no triangle (the reference reads face[1] regardless)
    const VertexRef i0 = face[0];
    VertexRef i1, i2 = face[1];
    for (size_t k = 2; k < face.size(); ++k) {
      i1 = i2;
      i2 = face[k];
      uint32_t a, b, c;
      if (!vertex(i0, &a) || !vertex(i1, &b) || !vertex(i2, &c)) return true;
      shape->indices.push_back(a);
      shape->indices.push_back(b);
      shape->indices.push_back(c);
      shape->material_ids.push_back(material);
    }
  }
  return true;
}

// LoadObj (tiny_obj_loader.cpp:780-1058).
std::string load_obj(const std::string& path, const std::string& base, ObjData* obj) {
  std::string text;
  if (!read_file(path, &text)) return "cannot open " + path;
  std::vector<std::vector<VertexRef>> group;
  Shape shape;
  int material = -1;
  std::string error;
  for_each_line(text, [&](const std::string& line) {
    if (!error.empty()) return;
    const char* t = line.c_str();
    t += std::strspn(t, " \t");
    if (t[0] == '\0' || t[0] == '#') return;
    if (t[0] == 'v' && is_blank(t[1])) {
      t += 2;
      for (int k = 0; k < 3; ++k) obj->v.push_back(parse_float(t));
    } else if (t[0] == 'v' && t[1] == 'n' && is_blank(t[2])) {
      t += 3;
      for (int k = 0; k < 3; ++k) obj->vn.push_back(parse_float(t));
    } else if (t[0] == 'v' && t[1] == 't' && is_blank(t[2])) {
      t += 3;
      for (int k = 0; k < 2; ++k) obj->vt.push_back(parse_float(t));
    } else if (t[0] == 'f' && is_blank(t[1])) {
      t += 2;
      t += std::strspn(t, " \t");
      std::vector<VertexRef> face;
      while (!is_line_end(t[0])) {
        face.push_back(parse_triple(t, (int)(obj->v.size() / 3), (int)(obj->vn.size() / 3), (int)(obj->vt.size() / 2)));
        t += std::strspn(t, " \t\r");
      }
      group.push_back(std::move(face));
    } else if (!std::strncmp(t, "usemtl", 6) && is_blank(t[6])) {
      const auto it = obj->material_map.find(first_word(t + 7));
      const int id = it == obj->material_map.end() ? -1 : it->second;
      if (id != material) {
        flush_group(*obj, group, material, &shape, &error);
        group.clear();
        material = id;
      }
    } else if (!std::strncmp(t, "mtllib", 6) && is_blank(t[6])) {
      load_mtl(base + first_word(t + 7), obj);
    } else if ((t[0] == 'g' || t[0] == 'o') && is_blank(t[1])) {
      if (flush_group(*obj, group, material, &shape, &error)) obj->shapes.push_back(std::move(shape));
      shape = Shape();
      group.clear();
    }
  });
  if (!error.empty()) return path + ": " + error;
  if (flush_group(*obj, group, material, &shape, &error)) obj->shapes.push_back(std::move(shape));
  if (!error.empty()) return path + ": " + error;
  return "";
}

struct V3 {
  float x, y, z;
};
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 normalized(V3 a) {
  const float d = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return {a.x / d, a.y / d, a.z / d};
}
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

int load_scene(const char* obj_file, const char* asset_dir, const char* environment_file, fr_material_fn material_fn,
               void* user, fr_scene* scene) {
  const std::string base = asset_dir ? asset_dir : "meshData//";
  ObjData obj;
  const std::string err = load_obj(obj_file, base, &obj);
  if (!err.empty()) return set_last_error(FR_ERR_IO, err);

  // Textures, loaded once per file name (AttributeManager::LoadTexture,
  // Normal_Facet.h:113-130); a name of two characters or fewer is not loaded
  // (Scene.cpp:41-56).
  std::map<std::string, int> texture_of;
  auto texture = [&](const std::string& name) -> int {
    if (name.size() <= 2) return -1;
    const std::string path = base + name;
    auto it = texture_of.find(path);
    if (it != texture_of.end()) return it->second;
    DecodedImage img;
    if (!decode_image_file(path, &img).empty()) return -1;  // the reference skips a texture it cannot load
    const int id = (int)scene->texels.size();
    scene->texels.push_back(std::move(img.rgba));
    scene->textures.push_back(fr_texture_desc{img.width, img.height, nullptr});
    texture_of[path] = id;
    return id;
  };
  std::vector<int> tex_kd(obj.materials.size()), tex_d(obj.materials.size()), tex_bump(obj.materials.size());
  for (size_t m = 0; m < obj.materials.size(); ++m) {
    tex_kd[m] = texture(obj.materials[m].map_kd);
    tex_d[m] = texture(obj.materials[m].map_d);
    tex_bump[m] = texture(obj.materials[m].map_bump);
  }

  // Attributes (Scene.cpp:60-77): SURFACE_PARAM() defaults, albedo Kd,
  // radiance Ke, then the material plug-in, then the textures.
  for (size_t m = 0; m < obj.materials.size(); ++m) {
    const MtlMaterial& mm = obj.materials[m];
    fr_material_desc d{};
    d.type = FR_MAT_DIFFUSE;
    d.sppm_surface = 0;
    d.opaque = 1;
    d.tex_albedo = d.tex_roughness = d.tex_bump = -1;
    for (int k = 0; k < 3; ++k) {
      d.albedo[k] = mm.kd[k];
      d.emission[k] = mm.ke[k];
    }
    d.index = 1.0f;
    d.roughness = 1.0f;
    d.extinction = 1.0f;
    d.reflectance = 1.0f;
    if (material_fn && material_fn(user, mm.name.c_str(), &d) != 0)
      return set_last_error(FR_ERR_INVALID, "material plug-in failed on material \"" + mm.name + "\"");
    d.tex_albedo = tex_kd[m];
    d.tex_roughness = tex_d[m];
    d.tex_bump = tex_bump[m];
    scene->materials.push_back(d);
    scene->material_names.push_back(mm.name);
  }

  // Facets (Scene.cpp:79-208).
  size_t total = 0;
  for (const Shape& s : obj.shapes) total += s.indices.size() / 3;
  if (total > 0x7FFFFFFF) return set_last_error(FR_ERR_INVALID, "too many facets");
  scene->positions.reserve(total * 9);
  scene->normals.reserve(total * 9);
  scene->uvs.reserve(total * 6);
  scene->material_ids.reserve(total);
  for (const Shape& s : obj.shapes) {
    for (size_t idx = 0, face = 0; idx + 2 < s.indices.size(); idx += 3, ++face) {
      V3 p[3];
      for (int k = 0; k < 3; ++k) {
        const size_t i = s.indices[idx + k];
        p[k] = V3{s.positions[3 * i], s.positions[3 * i + 1], s.positions[3 * i + 2]};
        scene->positions.insert(scene->positions.end(), {p[k].x, p[k].y, p[k].z});
      }
      if (!s.normals.empty()) {
        for (int k = 0; k < 3; ++k) {
          const size_t i = s.indices[idx + k];
          if (3 * i + 2 >= s.normals.size())
            return set_last_error(FR_ERR_IO, std::string(obj_file) +
                                                 ": a shape mixes vertices with and without normals (facet " +
                                                 std::to_string(scene->material_ids.size()) + ")");
          scene->normals.insert(scene->normals.end(), {s.normals[3 * i], s.normals[3 * i + 1], s.normals[3 * i + 2]});
        }
      } else {
        const V3 n = cross(normalized(sub(p[1], p[2])), normalized(sub(p[2], p[0])));
        for (int k = 0; k < 3; ++k) scene->normals.insert(scene->normals.end(), {n.x, n.y, n.z});
      }
      if (!s.texcoords.empty()) {
        for (int k = 0; k < 3; ++k) {
          const size_t i = s.indices[idx + k];
          if (2 * i + 1 >= s.texcoords.size())
            return set_last_error(FR_ERR_IO, std::string(obj_file) +
                                                 ": a shape mixes vertices with and without texture coordinates (facet " +
                                                 std::to_string(scene->material_ids.size()) + ")");
          scene->uvs.insert(scene->uvs.end(), {s.texcoords[2 * i], s.texcoords[2 * i + 1]});
        }
      } else {
        scene->uvs.insert(scene->uvs.end(), 6, 0.0f);
      }
      scene->material_ids.push_back(s.material_ids[face]);
    }
  }

  if (environment_file) {
    DecodedImage img;
    const std::string e = decode_image_file(environment_file, &img);
    if (!e.empty()) return set_last_error(FR_ERR_IO, e);
    scene->env_texels = std::move(img.rgba);
    scene->environment = fr_texture_desc{img.width, img.height, scene->env_texels.data()};
  }

  for (size_t i = 0; i < scene->textures.size(); ++i) scene->textures[i].texels = scene->texels[i].data();
  fr_scene_desc& d = scene->desc;
  d.num_facets = (int32_t)scene->material_ids.size();
  d.positions = scene->positions.data();
  d.normals = scene->normals.data();
  d.uvs = scene->uvs.data();
  d.material_ids = scene->material_ids.data();
  d.num_materials = (int32_t)scene->materials.size();
  d.materials = scene->materials.data();
  d.num_textures = (int32_t)scene->textures.size();
  d.textures = scene->textures.data();
  d.environment = environment_file ? &scene->environment : nullptr;
  return FR_OK;
}

}  // namespace
}  // namespace fr

extern "C" {

int fr_scene_load_obj(const char* obj_file, const char* asset_dir, const char* environment_file,
                      fr_material_fn material_fn, void* user, fr_scene** out) {
  if (!out) return fr::set_last_error(FR_ERR_INVALID, "fr_scene_load_obj: out is NULL");
  *out = nullptr;
  if (!obj_file) return fr::set_last_error(FR_ERR_INVALID, "fr_scene_load_obj: obj_file is NULL");
  fr_scene* scene = new fr_scene();
  const int rc = fr::load_scene(obj_file, asset_dir, environment_file, material_fn, user, scene);
  if (rc != FR_OK) {
    delete scene;
    return rc;
  }
  fr::set_last_error(FR_OK, "");
  *out = scene;
  return FR_OK;
}

const fr_scene_desc* fr_scene_get_desc(const fr_scene* scene) { return scene ? &scene->desc : nullptr; }

const char* fr_scene_material_name(const fr_scene* scene, int32_t m) {
  if (!scene || m < 0 || (size_t)m >= scene->material_names.size()) return nullptr;
  return scene->material_names[m].c_str();
}

void fr_scene_free(fr_scene* scene) { delete scene; }

}  // extern "C"
