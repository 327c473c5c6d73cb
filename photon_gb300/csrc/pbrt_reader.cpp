// pbrt-v4 reader: the reference's parse_pbrt_file
// (src/photon/pbrt/pbrt_parser.cpp:272-640, with ply_reader.cpp:62-251 and
// image_loader.cpp:20-106) and convert_pbrt_scene (pbrt_to_photon.cpp:58-503)
// in one pass, producing the renderer's phc_scene_desc with its
// path-tracer-level part (phc_pt_scene) instead of a Kokkos pt::Scene.
//
// The reference's reading of the format is kept where it departs from pbrt
// itself, because scenes must come out identical: numbers (integers
// included) go through strtof; a parameter's single unbracketed value is
// taken only for string/texture and float/integer/bool types; Transform sets
// the 16 values as given, Scale and Rotate multiply the flat row-major array
// on the right and ConcatTransform on the left; Translate, TransformBegin/End
// and unknown directives are read and ignored; Include paths are relative to
// the top-level file; instances take the transform current at ObjectInstance
// and are flattened (up to 500 per object and 5e8 triangles) unless
// use_instancing; normals are transformed with the matrix itself; an
// emissive shape gets its own emitter material.  All float arithmetic keeps
// the reference's operation order (the library compiles with
// -ffp-contract=off).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/photon_pbrt.h"

namespace phc {
void set_global_error(const std::string &msg);
}

namespace {

// ----------------------------------------------------------------- model
void identity16(float *m)
{
  for (int i = 0; i < 16; ++i)
    m[i] = (i % 5 == 0) ? 1.f : 0.f;
}

// r = a * b on flat row-major 4x4 arrays, summed from 0 in k order
void mul16(const float *a, const float *b, float *r)
{
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      float s = 0.f;
      for (int k = 0; k < 4; ++k)
        s += a[i * 4 + k] * b[k * 4 + j];
      r[i * 4 + j] = s;
    }
}

struct Vec3f {
  float x{0.f}, y{0.f}, z{0.f};
};

struct Mesh {
  std::vector<float> P, N, uv;
  std::vector<int> indices;
  std::string material, alpha_texture;
  Vec3f L;
  bool emissive{false};
  float xf[16];
};

struct NamedMaterial {
  std::string type;
  Vec3f reflectance{0.5f, 0.5f, 0.5f};
  Vec3f eta, k;
  float roughness{0.f}, uroughness{-1.f}, vroughness{-1.f}, eta_scalar{1.5f};
  std::string reflectance_texture;
};

struct Image {
  std::string class_type, filename;
  int width{0}, height{0};
  std::vector<float> rgb;
};

struct CameraDecl {
  float fov{45.f}, lensradius{0.f}, focaldistance{0.f};
  float xf[16];
  Vec3f from, at{0.f, 0.f, 1.f}, up{0.f, 1.f, 0.f};
  bool lookat{false};
};

struct Parsed {
  int width{512}, height{512}, spp{64}, max_depth{8};
  CameraDecl cam;
  std::map<std::string, Image> textures;
  std::map<std::string, NamedMaterial> materials;
  std::vector<Mesh> meshes;
  std::map<std::string, std::vector<Mesh>> objects;
  struct Placement {
    std::string object;
    float xf[16];
  };
  std::vector<Placement> instances; // every ObjectInstance of a defined object
  std::string env_file;
  float env_xf[16];
  float env_scale{1.f};
  bool has_env{false};
};

// ----------------------------------------------------------------- lexer
enum class Tk { Str, Num, LBr, RBr, Ident, End };
struct Token {
  Tk kind{Tk::End};
  std::string text;
  float num{0.f};
};

class Lexer {
public:
  explicit Lexer(const std::string &src) : p_(src.data()), end_(src.data() + src.size()) {}

  Token next()
  {
    for (;;) {
      while (p_ < end_) { // whitespace and # comments
        if (std::isspace(static_cast<unsigned char>(*p_)))
          ++p_;
        else if (*p_ == '#')
          while (p_ < end_ && *p_ != '\n')
            ++p_;
        else
          break;
      }
      if (p_ >= end_)
        return {};
      const char c = *p_;
      if (c == '[' || c == ']') {
        ++p_;
        return {c == '[' ? Tk::LBr : Tk::RBr, std::string(1, c), 0.f};
      }
      if (c == '"') {
        const char *s = ++p_;
        while (p_ < end_ && *p_ != '"')
          ++p_;
        Token t{Tk::Str, std::string(s, p_), 0.f};
        if (p_ < end_)
          ++p_;
        return t;
      }
      if (c == '-' || c == '+' || c == '.' || std::isdigit(static_cast<unsigned char>(c))) {
        const char *s = p_;
        if (c == '-' || c == '+')
          ++p_;
        while (p_ < end_ && (std::isdigit(static_cast<unsigned char>(*p_)) || *p_ == '.' || *p_ == 'e' ||
                                *p_ == 'E' || *p_ == '-' || *p_ == '+'))
          ++p_;
        Token t{Tk::Num, std::string(s, p_), 0.f};
        t.num = std::strtof(t.text.c_str(), nullptr);
        return t;
      }
      if (std::isalpha(static_cast<unsigned char>(c)) || c == '_') {
        const char *s = p_;
        while (p_ < end_ && (std::isalnum(static_cast<unsigned char>(*p_)) || *p_ == '_'))
          ++p_;
        return {Tk::Ident, std::string(s, p_), 0.f};
      }
      ++p_; // any other character is dropped
    }
  }

  Token peek()
  {
    const char *saved = p_;
    Token t = next();
    p_ = saved;
    return t;
  }

private:
  const char *p_, *end_;
};

// A "type name" parameter and its values.
struct Param {
  std::string type, name;
  std::vector<float> f;
  std::vector<int> i;
  std::vector<std::string> s;
};

bool int_type(const std::string &t) { return t == "integer" || t == "bool"; }

Param read_param(Lexer &lx)
{
  Param pv;
  const Token head = lx.next();
  if (head.kind != Tk::Str)
    return pv;
  const size_t sp = head.text.find(' ');
  if (sp == std::string::npos) {
    pv.name = head.text;
  } else {
    pv.type = head.text.substr(0, sp);
    pv.name = head.text.substr(sp + 1);
  }
  const Token v = lx.peek();
  if (v.kind == Tk::Str && (pv.type == "string" || pv.type == "texture")) {
    lx.next();
    pv.s.push_back(v.text);
    return pv;
  }
  if (v.kind == Tk::Num && (pv.type == "float" || int_type(pv.type))) {
    lx.next();
    if (int_type(pv.type))
      pv.i.push_back(int(v.num));
    else
      pv.f.push_back(v.num);
    return pv;
  }
  if (v.kind != Tk::LBr)
    return pv;
  lx.next();
  for (;;) {
    const Token e = lx.peek();
    if (e.kind == Tk::RBr) {
      lx.next();
      break;
    }
    if (e.kind == Tk::End)
      break;
    lx.next();
    if (e.kind == Tk::Num) {
      if (int_type(pv.type))
        pv.i.push_back(int(e.num));
      else
        pv.f.push_back(e.num);
    } else if (e.kind == Tk::Str) {
      pv.s.push_back(e.text);
    }
  }
  return pv;
}

// Reads every parameter that follows a directive.
template <class F> void each_param(Lexer &lx, F &&f)
{
  while (lx.peek().kind == Tk::Str)
    f(read_param(lx));
}

void skip_params(Lexer &lx)
{
  each_param(lx, [](const Param &) {});
}

// sRGB stand-ins of measured metal spectra (pbrt_parser.cpp:183-195)
Vec3f named_spectrum(const std::string &n)
{
  static const struct {
    const char *name;
    Vec3f v;
  } table[] = {
      {"metal-Ag-eta", {0.155f, 0.116f, 0.138f}}, {"metal-Ag-k", {4.828f, 3.122f, 2.146f}},
      {"metal-Au-eta", {0.143f, 0.374f, 1.442f}}, {"metal-Au-k", {3.983f, 2.387f, 1.603f}},
      {"metal-Cu-eta", {0.200f, 0.924f, 1.102f}}, {"metal-Cu-k", {3.912f, 2.452f, 2.142f}},
      {"metal-Al-eta", {1.345f, 0.965f, 0.612f}}, {"metal-Al-k", {7.474f, 6.400f, 5.275f}},
      {"metal-Fe-eta", {2.912f, 2.950f, 2.584f}}, {"metal-Fe-k", {3.070f, 2.930f, 2.771f}},
  };
  for (const auto &e : table)
    if (n == e.name)
      return e.v;
  return {};
}

// ----------------------------------------------------------------- files
std::string dir_of(const std::string &path)
{
  const size_t s = path.find_last_of("/\\");
  return s == std::string::npos ? std::string() : path.substr(0, s + 1);
}

// Inlines Include/Import lines (paths relative to the top-level file's
// directory), ten levels deep at most (pbrt_parser.cpp:242-270).
std::string expand_includes(const std::string &path, const std::string &root, int depth)
{
  if (depth > 10)
    return {};
  std::ifstream f(path);
  if (!f.is_open()) {
    std::fprintf(stderr, "  Warning: cannot open %s\n", path.c_str());
    return {};
  }
  std::string out, line;
  while (std::getline(f, line)) {
    std::string t = line;
    const size_t b = t.find_first_not_of(" \t");
    if (b != std::string::npos)
      t = t.substr(b);
    if (t.size() > 5 && (t.compare(0, 7, "Include") == 0 || t.compare(0, 6, "Import") == 0)) {
      const size_t q1 = t.find('"'), q2 = t.rfind('"');
      if (q1 != std::string::npos && q2 > q1) {
        out += expand_includes(root + t.substr(q1 + 1, q2 - q1 - 1), root, depth + 1);
        continue;
      }
    }
    out += line;
    out += '\n';
  }
  return out;
}

// PLY property type sizes and integer reads (ply_reader.cpp:30-59): types
// that are not listed read as 4-byte ints.
int ply_size(const std::string &t)
{
  if (t == "float" || t == "float32" || t == "int" || t == "int32" || t == "uint" || t == "uint32")
    return 4;
  if (t == "double" || t == "float64" || t == "int64" || t == "uint64")
    return 8;
  if (t == "uchar" || t == "uint8" || t == "char" || t == "int8")
    return 1;
  if (t == "short" || t == "int16" || t == "ushort" || t == "uint16")
    return 2;
  return 4;
}

template <class T> T read_raw(std::istream &in)
{
  T v{};
  in.read(reinterpret_cast<char *>(&v), sizeof(T));
  return v;
}

int ply_int(std::istream &in, const std::string &t)
{
  if (t == "uchar" || t == "uint8")
    return int(read_raw<uint8_t>(in));
  if (t == "uint" || t == "uint32")
    return int(read_raw<uint32_t>(in));
  if (t == "short" || t == "int16")
    return int(read_raw<int16_t>(in));
  if (t == "ushort" || t == "uint16")
    return int(read_raw<uint16_t>(in));
  return int(read_raw<int32_t>(in));
}

struct PlyProp {
  std::string name, type, count_type, value_type;
  bool list{false};
};
struct PlyElem {
  std::string name;
  int count{0};
  std::vector<PlyProp> props;
};

bool load_ply(const std::string &path, Mesh &mesh)
{
  std::ifstream in(path, std::ios::binary);
  if (!in.is_open()) {
    std::fprintf(stderr, "PLY: cannot open %s\n", path.c_str());
    return false;
  }
  std::string line;
  std::getline(in, line);
  if (line.find("ply") == std::string::npos) {
    std::fprintf(stderr, "PLY: not a PLY file: %s\n", path.c_str());
    return false;
  }
  enum { ASCII, LE, BE } fmt = LE;
  std::vector<PlyElem> elems;
  while (std::getline(in, line)) {
    if (line.empty() || line[0] == '\r')
      continue;
    if (line.back() == '\r')
      line.pop_back();
    std::istringstream ss(line);
    std::string kw;
    ss >> kw;
    if (kw == "end_header")
      break;
    if (kw == "format") {
      std::string f;
      ss >> f;
      if (f == "ascii")
        fmt = ASCII;
      else if (f == "binary_big_endian")
        fmt = BE;
    } else if (kw == "element") {
      PlyElem e;
      ss >> e.name >> e.count;
      elems.push_back(e);
    } else if (kw == "property" && !elems.empty()) {
      PlyProp p;
      std::string w;
      ss >> w;
      if (w == "list") {
        p.list = true;
        ss >> p.count_type >> p.value_type >> p.name;
      } else {
        p.type = w;
        ss >> p.name;
      }
      elems.back().props.push_back(p);
    }
  }
  if (fmt == BE) {
    std::fprintf(stderr, "PLY: big-endian not supported: %s\n", path.c_str());
    return false;
  }
  int vi_el = -1, fi_el = -1;
  for (int i = 0; i < int(elems.size()); ++i) {
    if (elems[i].name == "vertex")
      vi_el = i;
    if (elems[i].name == "face")
      fi_el = i;
  }
  if (vi_el < 0 || fi_el < 0) {
    std::fprintf(stderr, "PLY: missing vertex or face element: %s\n", path.c_str());
    return false;
  }
  const PlyElem &ve = elems[size_t(vi_el)], &fe = elems[size_t(fi_el)];
  int px = -1, py = -1, pz = -1, nx = -1, ny = -1, nz = -1, pu = -1, pv = -1;
  for (int i = 0; i < int(ve.props.size()); ++i) {
    const std::string &n = ve.props[size_t(i)].name;
    if (n == "x")
      px = i;
    else if (n == "y")
      py = i;
    else if (n == "z")
      pz = i;
    else if (n == "nx")
      nx = i;
    else if (n == "ny")
      ny = i;
    else if (n == "nz")
      nz = i;
    else if (n == "u" || n == "s" || n == "texture_u")
      pu = i;
    else if (n == "v" || n == "t" || n == "texture_v")
      pv = i;
  }
  const bool has_n = nx >= 0 && ny >= 0 && nz >= 0, has_uv = pu >= 0 && pv >= 0;
  const size_t nv = size_t(std::max(ve.count, 0));
  mesh.P.assign(nv * 3, 0.f);
  if (has_n)
    mesh.N.assign(nv * 3, 0.f);
  if (has_uv)
    mesh.uv.assign(nv * 2, 0.f);
  std::vector<float> vals(std::max<size_t>(ve.props.size(), 16));
  auto store = [&](size_t v) {
    if (px >= 0)
      mesh.P[v * 3] = vals[size_t(px)];
    if (py >= 0)
      mesh.P[v * 3 + 1] = vals[size_t(py)];
    if (pz >= 0)
      mesh.P[v * 3 + 2] = vals[size_t(pz)];
    if (has_n) {
      mesh.N[v * 3] = vals[size_t(nx)];
      mesh.N[v * 3 + 1] = vals[size_t(ny)];
      mesh.N[v * 3 + 2] = vals[size_t(nz)];
    }
    if (has_uv) {
      mesh.uv[v * 2] = vals[size_t(pu)];
      mesh.uv[v * 2 + 1] = vals[size_t(pv)];
    }
  };
  auto fan = [&](const std::vector<int> &f) {
    for (size_t j = 1; j + 1 < f.size(); ++j) {
      mesh.indices.push_back(f[0]);
      mesh.indices.push_back(f[j]);
      mesh.indices.push_back(f[j + 1]);
    }
  };
  std::vector<int> face;
  if (fmt == LE) {
    for (size_t v = 0; v < nv; ++v) {
      std::fill(vals.begin(), vals.end(), 0.f);
      for (size_t k = 0; k < ve.props.size(); ++k) {
        const PlyProp &p = ve.props[k];
        if (p.type == "float" || p.type == "float32")
          vals[k] = read_raw<float>(in);
        else
          in.seekg(ply_size(p.type), std::ios::cur);
      }
      store(v);
    }
    for (int f = 0; f < fe.count; ++f)
      for (const PlyProp &p : fe.props) {
        if (p.list && (p.name == "vertex_indices" || p.name == "vertex_index")) {
          const int n = ply_int(in, p.count_type);
          face.assign(size_t(std::max(n, 0)), 0);
          for (int j = 0; j < n; ++j)
            face[size_t(j)] = ply_int(in, p.value_type);
          fan(face);
        } else if (p.list) {
          const int n = ply_int(in, p.count_type);
          for (int j = 0; j < n; ++j)
            in.seekg(ply_size(p.value_type), std::ios::cur);
        } else {
          in.seekg(ply_size(p.type), std::ios::cur);
        }
      }
  } else {
    for (size_t v = 0; v < nv; ++v) {
      for (size_t k = 0; k < ve.props.size(); ++k) {
        float x = 0.f;
        in >> x;
        vals[k] = x;
      }
      store(v);
    }
    for (int f = 0; f < fe.count; ++f) {
      int n = 0;
      in >> n;
      face.assign(size_t(std::max(n, 0)), 0);
      for (int j = 0; j < n; ++j)
        in >> face[size_t(j)];
      fan(face);
    }
  }
  return !mesh.P.empty() && !mesh.indices.empty();
}

// PFM, rows stored bottom-up, read into top-down order (image_loader.cpp:
// 20-74); 1-channel images replicate to RGB.
bool load_pfm(const std::string &path, Image &img)
{
  std::ifstream in(path, std::ios::binary);
  if (!in.is_open())
    return false;
  std::string magic, dims, scale_line;
  std::getline(in, magic);
  if (magic != "PF" && magic != "Pf")
    return false;
  const int ch = magic == "PF" ? 3 : 1;
  std::getline(in, dims);
  int w = 0, h = 0;
  std::sscanf(dims.c_str(), "%d %d", &w, &h);
  if (w <= 0 || h <= 0)
    return false;
  std::getline(in, scale_line);
  float scale = 0.f;
  std::sscanf(scale_line.c_str(), "%f", &scale);
  float s = std::fabs(scale);
  if (s == 0.f)
    s = 1.f;
  img.width = w;
  img.height = h;
  img.rgb.assign(size_t(w) * size_t(h) * 3, 0.f);
  std::vector<float> row(size_t(w) * size_t(ch), 0.f);
  for (int y = h - 1; y >= 0; --y) {
    in.read(reinterpret_cast<char *>(row.data()), std::streamsize(row.size() * sizeof(float)));
    for (int x = 0; x < w; ++x) {
      float *d = &img.rgb[(size_t(y) * size_t(w) + size_t(x)) * 3];
      if (ch == 3) {
        d[0] = row[size_t(x) * 3] * s;
        d[1] = row[size_t(x) * 3 + 1] * s;
        d[2] = row[size_t(x) * 3 + 2] * s;
      } else {
        d[0] = d[1] = d[2] = row[size_t(x)] * s;
      }
    }
  }
  return true;
}

bool load_image(const std::string &path, Image &img)
{
  if (path.size() >= 4) {
    std::string ext = path.substr(path.size() - 4);
    for (char &c : ext)
      c = char(std::tolower(static_cast<unsigned char>(c)));
    if (ext == ".pfm")
      return load_pfm(path, img);
  }
  std::fprintf(stderr, "Warning: cannot load texture: %s (PFM only)\n", path.c_str());
  return false;
}

// ---------------------------------------------------------------- parser
struct GState {
  std::string material;
  float xf[16];
  Vec3f L;
  bool area{false};
};

constexpr uint64_t kMaxInstancesPerObject = 500;     // pbrt_scene.h:89
constexpr uint64_t kMaxTotalTriangles = 500000000ull; // pbrt_scene.h:90

void tessellate_sphere(float radius, Mesh &m)
{
  const int slices = 32, stacks = 16;
  for (int j = 0; j <= stacks; ++j) {
    const float theta = (float(j) / float(stacks)) * 3.14159265f;
    const float st = std::sin(theta), ct = std::cos(theta);
    for (int i = 0; i <= slices; ++i) {
      const float phi = (float(i) / float(slices)) * 6.28318530f;
      m.P.push_back(st * std::cos(phi) * radius);
      m.P.push_back(ct * radius);
      m.P.push_back(st * std::sin(phi) * radius);
      m.N.push_back(st * std::cos(phi));
      m.N.push_back(ct);
      m.N.push_back(st * std::sin(phi));
    }
  }
  for (int j = 0; j < stacks; ++j)
    for (int i = 0; i < slices; ++i) {
      const int a = j * (slices + 1) + i, b = a + 1, c = a + slices + 1, d = c + 1;
      const int tri[6] = {a, c, b, b, c, d};
      m.indices.insert(m.indices.end(), tri, tri + 6);
    }
}

Parsed parse(const std::string &path, bool use_instancing)
{
  const std::string base = dir_of(path);
  const std::string text = expand_includes(path, base, 0);
  Lexer lx(text);
  Parsed sc;
  identity16(sc.cam.xf);
  identity16(sc.env_xf);
  std::vector<GState> stack;
  GState st;
  identity16(st.xf);
  std::string object;
  std::map<std::string, uint64_t> inst_count;
  uint64_t total_tris = 0;

  auto new_mesh = [&](Mesh &m) {
    m.material = st.material;
    std::memcpy(m.xf, st.xf, sizeof(m.xf));
    if (st.area) {
      m.emissive = true;
      m.L = st.L;
    }
  };
  auto add_mesh = [&](Mesh &&m) {
    if (!object.empty()) {
      sc.objects[object].push_back(std::move(m));
    } else {
      total_tris += m.indices.size() / 3;
      sc.meshes.push_back(std::move(m));
    }
  };
  auto post_multiply = [&](const float *m) {
    float r[16];
    mul16(st.xf, m, r);
    std::memcpy(st.xf, r, sizeof(r));
  };

  for (;;) {
    const Token t = lx.next();
    if (t.kind == Tk::End)
      break;
    if (t.kind != Tk::Ident)
      continue;
    const std::string &d = t.text;
    if (d == "Integrator") {
      lx.next();
      each_param(lx, [&](const Param &p) {
        if (p.name == "maxdepth" && !p.i.empty())
          sc.max_depth = p.i[0];
      });
    } else if (d == "Sampler") {
      lx.next();
      each_param(lx, [&](const Param &p) {
        if (p.name == "pixelsamples" && !p.i.empty())
          sc.spp = p.i[0];
      });
    } else if (d == "Film") {
      lx.next();
      each_param(lx, [&](const Param &p) {
        if (p.name == "xresolution" && !p.i.empty())
          sc.width = p.i[0];
        else if (p.name == "yresolution" && !p.i.empty())
          sc.height = p.i[0];
      });
    } else if (d == "PixelFilter") {
      lx.next();
      skip_params(lx);
    } else if (d == "Camera") {
      lx.next();
      std::memcpy(sc.cam.xf, st.xf, sizeof(st.xf));
      each_param(lx, [&](const Param &p) {
        if (p.name == "fov" && !p.f.empty())
          sc.cam.fov = p.f[0];
        else if (p.name == "lensradius" && !p.f.empty())
          sc.cam.lensradius = p.f[0];
        else if (p.name == "focaldistance" && !p.f.empty())
          sc.cam.focaldistance = p.f[0];
      });
    } else if (d == "Transform") {
      if (lx.next().kind == Tk::LBr) {
        for (int i = 0; i < 16; ++i)
          st.xf[i] = lx.next().num;
        lx.next();
      }
    } else if (d == "LookAt") {
      float v[9];
      for (float &x : v)
        x = lx.next().num;
      sc.cam.from = {v[0], v[1], v[2]};
      sc.cam.at = {v[3], v[4], v[5]};
      sc.cam.up = {v[6], v[7], v[8]};
      sc.cam.lookat = true;
    } else if (d == "Scale") {
      const float sx = lx.next().num, sy = lx.next().num, sz = lx.next().num;
      const float s[16] = {sx, 0, 0, 0, 0, sy, 0, 0, 0, 0, sz, 0, 0, 0, 0, 1};
      post_multiply(s);
    } else if (d == "Rotate") {
      const float angle = lx.next().num;
      float ax = lx.next().num, ay = lx.next().num, az = lx.next().num;
      const float len = std::sqrt(ax * ax + ay * ay + az * az);
      if (len > 0.f) {
        ax /= len;
        ay /= len;
        az /= len;
      }
      const float rad = angle * 3.14159265f / 180.f;
      const float c = std::cos(rad), s = std::sin(rad), u = 1.f - c;
      const float r[16] = {u * ax * ax + c, u * ax * ay - s * az, u * ax * az + s * ay, 0,
          u * ax * ay + s * az, u * ay * ay + c, u * ay * az - s * ax, 0,
          u * ax * az - s * ay, u * ay * az + s * ax, u * az * az + c, 0, 0, 0, 0, 1};
      post_multiply(r);
    } else if (d == "ConcatTransform") {
      if (lx.next().kind == Tk::LBr) {
        float m[16], r[16];
        for (float &x : m)
          x = lx.next().num;
        lx.next();
        mul16(m, st.xf, r); // pre-multiplied, as the reference does
        std::memcpy(st.xf, r, sizeof(r));
      }
    } else if (d == "Identity") {
      identity16(st.xf);
    } else if (d == "WorldBegin") {
      identity16(st.xf);
    } else if (d == "AttributeBegin") {
      stack.push_back(st);
    } else if (d == "AttributeEnd") {
      if (!stack.empty()) {
        st = stack.back();
        stack.pop_back();
      }
    } else if (d == "MakeNamedMaterial") {
      const std::string name = lx.next().text;
      NamedMaterial m;
      each_param(lx, [&](const Param &p) {
        if (p.name == "type" && !p.s.empty())
          m.type = p.s[0];
        else if (p.name == "reflectance" && p.type == "texture" && !p.s.empty())
          m.reflectance_texture = p.s[0];
        else if (p.name == "reflectance" && p.f.size() >= 3)
          m.reflectance = {p.f[0], p.f[1], p.f[2]};
        else if (p.name == "roughness" && !p.f.empty())
          m.roughness = p.f[0];
        else if (p.name == "eta") {
          if (!p.s.empty())
            m.eta = named_spectrum(p.s[0]);
          else if (p.f.size() >= 3)
            m.eta = {p.f[0], p.f[1], p.f[2]};
          else if (p.f.size() == 1)
            m.eta_scalar = p.f[0];
        } else if (p.name == "k") {
          if (!p.s.empty())
            m.k = named_spectrum(p.s[0]);
          else if (p.f.size() >= 3)
            m.k = {p.f[0], p.f[1], p.f[2]};
        } else if (p.name == "uroughness" && !p.f.empty())
          m.uroughness = p.f[0];
        else if (p.name == "vroughness" && !p.f.empty())
          m.vroughness = p.f[0];
      });
      sc.materials[name] = m;
    } else if (d == "NamedMaterial") {
      st.material = lx.next().text;
    } else if (d == "AreaLightSource") {
      lx.next();
      st.area = true;
      each_param(lx, [&](const Param &p) {
        if (p.name == "L" && p.f.size() >= 3)
          st.L = {p.f[0], p.f[1], p.f[2]};
      });
    } else if (d == "Shape") {
      const std::string type = lx.next().text;
      if (type == "trianglemesh") {
        Mesh m;
        new_mesh(m);
        each_param(lx, [&](const Param &p) {
          if ((p.name == "P" || p.name == "p") && p.type == "point3")
            m.P = p.f;
          else if (p.name == "indices" && p.type == "integer")
            m.indices = p.i;
          else if (p.name == "N" && p.type == "normal")
            m.N = p.f;
          else if (p.name == "uv" && p.type == "point2")
            m.uv = p.f;
        });
        if (!m.P.empty() && !m.indices.empty())
          add_mesh(std::move(m));
      } else if (type == "plymesh") {
        Mesh m;
        new_mesh(m);
        std::string file;
        each_param(lx, [&](const Param &p) {
          if (p.name == "filename" && !p.s.empty())
            file = p.s[0];
          else if (p.name == "alpha" && p.type == "texture" && !p.s.empty())
            m.alpha_texture = p.s[0];
        });
        if (!file.empty()) {
          if (load_ply(base + file, m))
            add_mesh(std::move(m));
          else
            std::fprintf(stderr, "Warning: failed to load PLY: %s\n", (base + file).c_str());
        }
      } else if (type == "sphere") {
        Mesh m;
        new_mesh(m);
        float radius = 1.f;
        each_param(lx, [&](const Param &p) {
          if (p.name == "radius" && !p.f.empty())
            radius = p.f[0];
        });
        tessellate_sphere(radius, m);
        add_mesh(std::move(m));
      } else {
        skip_params(lx);
      }
    } else if (d == "Texture") {
      const std::string name = lx.next().text;
      lx.next(); // value type
      Image img;
      img.class_type = lx.next().text;
      each_param(lx, [&](const Param &p) {
        if (p.name == "filename" && !p.s.empty())
          img.filename = p.s[0];
      });
      sc.textures[name] = img;
    } else if (d == "LightSource") {
      const std::string type = lx.next().text;
      if (type == "infinite") {
        sc.has_env = true;
        std::memcpy(sc.env_xf, st.xf, sizeof(st.xf));
        each_param(lx, [&](const Param &p) {
          if (p.name == "filename" && !p.s.empty())
            sc.env_file = p.s[0];
          else if ((p.name == "scale" || p.name == "L") && p.f.size() >= 3)
            sc.env_scale = (p.f[0] + p.f[1] + p.f[2]) / 3.f;
        });
      } else {
        skip_params(lx);
      }
    } else if (d == "ObjectBegin") {
      object = lx.next().text;
    } else if (d == "ObjectEnd") {
      object.clear();
    } else if (d == "ObjectInstance") {
      const std::string name = lx.next().text;
      const auto it = sc.objects.find(name);
      if (it == sc.objects.end())
        continue;
      Parsed::Placement pl;
      pl.object = name;
      std::memcpy(pl.xf, st.xf, sizeof(st.xf));
      sc.instances.push_back(pl);
      if (use_instancing || total_tris >= kMaxTotalTriangles)
        continue;
      uint64_t &count = inst_count[name];
      if (count >= kMaxInstancesPerObject)
        continue;
      uint64_t obj_tris = 0;
      for (const Mesh &m : it->second)
        obj_tris += m.indices.size() / 3;
      if (total_tris + obj_tris > kMaxTotalTriangles)
        continue;
      for (const Mesh &om : it->second) {
        Mesh m = om;
        std::memcpy(m.xf, st.xf, sizeof(st.xf));
        sc.meshes.push_back(std::move(m));
      }
      total_tris += obj_tris;
      ++count;
    } else if (d == "Material" || d == "MakeNamedMedium") {
      lx.next();
      skip_params(lx);
    } else if (d == "ReverseOrientation" || d == "TransformBegin" || d == "TransformEnd" ||
               d == "MediumInterface") {
      skip_params(lx);
    }
  }
  return sc;
}

// ------------------------------------------------------------- converter
struct Mat4 {
  float m[4][4]{};
};

// pbrt matrices are column-major (pbrt_to_photon.cpp:23-30)
Mat4 from_column_major(const float *cm)
{
  Mat4 r;
  for (int c = 0; c < 4; ++c)
    for (int row = 0; row < 4; ++row)
      r.m[row][c] = cm[c * 4 + row];
  return r;
}

// Mat4::transform_point / transform_direction / inverse
// (include/photon/pt/math_mat4.h:77-144)
Vec3f xf_point(const Mat4 &a, const Vec3f &p)
{
  const auto &m = a.m;
  const float x = m[0][0] * p.x + m[0][1] * p.y + m[0][2] * p.z + m[0][3];
  const float y = m[1][0] * p.x + m[1][1] * p.y + m[1][2] * p.z + m[1][3];
  const float z = m[2][0] * p.x + m[2][1] * p.y + m[2][2] * p.z + m[2][3];
  const float w = m[3][0] * p.x + m[3][1] * p.y + m[3][2] * p.z + m[3][3];
  if (w != 0.f && w != 1.f) {
    const float iw = 1.f / w;
    return {x * iw, y * iw, z * iw};
  }
  return {x, y, z};
}

Vec3f xf_dir(const Mat4 &a, const Vec3f &d)
{
  const auto &m = a.m;
  return {m[0][0] * d.x + m[0][1] * d.y + m[0][2] * d.z, m[1][0] * d.x + m[1][1] * d.y + m[1][2] * d.z,
      m[2][0] * d.x + m[2][1] * d.y + m[2][2] * d.z};
}

Mat4 inverse(const Mat4 &a)
{
  const auto &m = a.m;
  Mat4 r;
  for (int i = 0; i < 4; ++i)
    r.m[i][i] = 1.f;
  const float a00 = m[0][0], a01 = m[0][1], a02 = m[0][2];
  const float a10 = m[1][0], a11 = m[1][1], a12 = m[1][2];
  const float a20 = m[2][0], a21 = m[2][1], a22 = m[2][2];
  const float det = a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) + a02 * (a10 * a21 - a11 * a20);
  if (det == 0.f)
    return Mat4{};
  const float id = 1.f / det;
  r.m[0][0] = (a11 * a22 - a12 * a21) * id;
  r.m[0][1] = (a02 * a21 - a01 * a22) * id;
  r.m[0][2] = (a01 * a12 - a02 * a11) * id;
  r.m[1][0] = (a12 * a20 - a10 * a22) * id;
  r.m[1][1] = (a00 * a22 - a02 * a20) * id;
  r.m[1][2] = (a02 * a10 - a00 * a12) * id;
  r.m[2][0] = (a10 * a21 - a11 * a20) * id;
  r.m[2][1] = (a01 * a20 - a00 * a21) * id;
  r.m[2][2] = (a00 * a11 - a01 * a10) * id;
  const float tx = m[0][3], ty = m[1][3], tz = m[2][3];
  r.m[0][3] = -(r.m[0][0] * tx + r.m[0][1] * ty + r.m[0][2] * tz);
  r.m[1][3] = -(r.m[1][0] * tx + r.m[1][1] * ty + r.m[1][2] * tz);
  r.m[2][3] = -(r.m[2][0] * tx + r.m[2][1] * ty + r.m[2][2] * tz);
  return r;
}

Vec3f sub(const Vec3f &a, const Vec3f &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
Vec3f cross3(const Vec3f &a, const Vec3f &b)
{
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
float length3(const Vec3f &v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
Vec3f normalize3(const Vec3f &v)
{
  const float l = length3(v);
  if (!(l > 0.f))
    return {};
  const float il = 1.f / l;
  return {v.x * il, v.y * il, v.z * il};
}

phc_pt_material default_pt_material() // pt::Material{} (material.h:35-82)
{
  phc_pt_material m{};
  m.base_color[0] = m.base_color[1] = m.base_color[2] = 0.8f;
  m.metallic = 0.f;
  m.roughness = 0.5f;
  m.ior = 1.5f;
  m.transmission = 0.f;
  m.specular = 0.5f;
  m.clearcoat = 0.f;
  m.clearcoat_roughness = 0.03f;
  m.sheen = 0.f;
  m.alpha = 1.f;
  m.emission_strength = 0.f;
  m.flags = 0;
  m.base_color_tex = -1;
  m.alpha_tex = -1;
  return m;
}

void set3(float *d, float x, float y, float z)
{
  d[0] = x;
  d[1] = y;
  d[2] = z;
}

// The float that the renderer turns back into `deg` degrees: the bridge
// computes fovy * 180 / pi (RenderBridge.cpp:872-891), so pick the radian
// value whose conversion reproduces the file's fov exactly when one exists.
float fovy_for_degrees(float deg)
{
  const float guess = deg * 3.14159265358979f / 180.f;
  float best = guess, best_err = 1e30f;
  float v = guess;
  for (int k = 0; k < 8; ++k)
    v = std::nextafter(v, -1e30f);
  for (int k = 0; k < 17; ++k, v = std::nextafter(v, 1e30f)) {
    const float back = v * 180.f / 3.14159265358979f;
    const float err = std::fabs(back - deg);
    if (err < best_err) {
      best_err = err;
      best = v;
    }
    if (back == deg)
      return v;
  }
  return best;
}

} // namespace

struct phc_pbrt_scene {
  // converted geometry (flattened: three vertices per triangle)
  std::vector<float> positions, normals, texcoords;
  std::vector<uint32_t> indices, material_ids;
  std::vector<phc_pt_material> materials;
  std::vector<std::vector<float>> texture_pixels;
  std::vector<phc_texture> textures;
  std::vector<float> env_pixels;
  // instanced geometry (use_instancing): merged objects and placements
  struct ObjectData {
    std::vector<float> positions, normals;
    std::vector<uint32_t> indices;
  };
  std::vector<ObjectData> object_data;
  std::vector<phc_object> objects;
  std::vector<phc_instance> instances;
  phc_pt_scene pt{};
  phc_scene_desc desc{};
  phc_camera camera{};
  phc_settings settings{};
  phc_pbrt_info info{};
};

namespace {

void convert(const Parsed &ps, const std::string &base, bool use_instancing, phc_pbrt_scene &out)
{
  // textures: every imagemap with a file name is loaded; the atlas holds the
  // loaded ones in name order (pbrt_to_photon.cpp:62-90)
  std::map<std::string, Image> textures = ps.textures;
  for (auto &kv : textures) {
    Image &t = kv.second;
    if (t.class_type == "imagemap" && !t.filename.empty() && t.rgb.empty())
      load_image(base + t.filename, t);
  }
  std::map<std::string, int32_t> tex_id;
  for (const auto &kv : textures) {
    const Image &t = kv.second;
    if (!t.rgb.empty() && t.width > 0 && t.height > 0) {
      tex_id[kv.first] = int32_t(out.textures.size());
      out.texture_pixels.push_back(t.rgb);
      phc_texture td{};
      td.width = uint32_t(t.width);
      td.height = uint32_t(t.height);
      out.textures.push_back(td);
    }
  }
  for (size_t i = 0; i < out.textures.size(); ++i)
    out.textures[i].rgb = out.texture_pixels[i].data();

  // named materials in name order (pbrt_to_photon.cpp:98-170)
  std::map<std::string, uint32_t> mat_id;
  for (const auto &kv : ps.materials) {
    const NamedMaterial &pm = kv.second;
    mat_id[kv.first] = uint32_t(out.materials.size());
    phc_pt_material m = default_pt_material();
    if (!pm.reflectance_texture.empty()) {
      const auto it = tex_id.find(pm.reflectance_texture);
      if (it != tex_id.end())
        m.base_color_tex = it->second;
    }
    const Vec3f &rf = pm.reflectance;
    auto uv_roughness = [&pm] {
      float r = pm.roughness;
      if (pm.uroughness >= 0.f)
        r = (pm.uroughness + (pm.vroughness >= 0.f ? pm.vroughness : pm.uroughness)) * 0.5f;
      return r;
    };
    if (pm.type == "diffuse") {
      set3(m.base_color, rf.x, rf.y, rf.z);
      m.roughness = 1.f;
      m.metallic = 0.f;
    } else if (pm.type == "conductor") {
      auto f0 = [](float eta, float k) {
        const float num = (eta - 1.f) * (eta - 1.f) + k * k;
        const float den = (eta + 1.f) * (eta + 1.f) + k * k;
        return den > 0.f ? num / den : 0.f;
      };
      set3(m.base_color, f0(pm.eta.x, pm.k.x), f0(pm.eta.y, pm.k.y), f0(pm.eta.z, pm.k.z));
      m.metallic = 1.f;
      m.roughness = uv_roughness();
    } else if (pm.type == "dielectric") {
      set3(m.base_color, 1.f, 1.f, 1.f);
      m.ior = pm.eta_scalar;
      m.transmission = 1.f;
      m.roughness = uv_roughness();
    } else if (pm.type == "coateddiffuse") {
      set3(m.base_color, rf.x, rf.y, rf.z);
      m.metallic = 0.f;
      const float r = uv_roughness();
      m.roughness = r;
      m.clearcoat = 1.f;
      m.clearcoat_roughness = r * 0.5f;
    } else if (pm.type == "diffusetransmission") {
      set3(m.base_color, rf.x, rf.y, rf.z);
      m.roughness = 1.f;
      m.metallic = 0.f;
      m.transmission = 0.5f;
    } else {
      set3(m.base_color, rf.x, rf.y, rf.z);
      m.roughness = pm.roughness;
    }
    out.materials.push_back(m);
  }
  if (out.materials.empty()) {
    phc_pt_material m = default_pt_material();
    set3(m.base_color, 0.5f, 0.5f, 0.5f);
    m.roughness = 1.f;
    out.materials.push_back(m);
  }

  // meshes, flattened into world space (pbrt_to_photon.cpp:172-277)
  uint64_t total = 0;
  for (const Mesh &mesh : ps.meshes)
    total += mesh.indices.size() / 3;
  if (total * 3 > 0xffffffffull)
    throw std::length_error("pbrt: more than 2^32 flattened vertices");
  out.positions.reserve(total * 9);
  out.normals.reserve(total * 9);
  out.texcoords.assign(total * 6, 0.f);
  out.material_ids.reserve(total);
  uint64_t emissive = 0;
  for (const Mesh &mesh : ps.meshes) {
    const Mat4 xf = from_column_major(mesh.xf);
    uint32_t mid = 0;
    const auto it = mat_id.find(mesh.material);
    if (it != mat_id.end())
      mid = it->second;
    const size_t nverts = mesh.P.size() / 3;
    const bool has_uv = mesh.uv.size() >= nverts * 2;
    if (!mesh.alpha_texture.empty()) {
      const auto at = tex_id.find(mesh.alpha_texture);
      if (at != tex_id.end()) {
        phc_pt_material am = out.materials[mid];
        am.alpha_tex = at->second;
        mid = uint32_t(out.materials.size());
        out.materials.push_back(am);
      }
    }
    if (mesh.emissive) {
      phc_pt_material em = default_pt_material();
      set3(em.base_color, 0.f, 0.f, 0.f);
      set3(em.emission, mesh.L.x, mesh.L.y, mesh.L.z);
      em.emission_strength = 1.f;
      em.roughness = 1.f;
      mid = uint32_t(out.materials.size());
      out.materials.push_back(em);
    }
    const bool has_n = mesh.N.size() >= mesh.P.size();
    const size_t ntris = mesh.indices.size() / 3;
    for (size_t t = 0; t < ntris; ++t) {
      int idx[3];
      Vec3f p[3];
      for (int k = 0; k < 3; ++k) {
        idx[k] = mesh.indices[3 * t + size_t(k)];
        if (idx[k] < 0 || size_t(idx[k]) >= nverts)
          throw std::out_of_range("pbrt: vertex index out of range in a shape");
        const size_t v = size_t(idx[k]);
        p[k] = xf_point(xf, {mesh.P[3 * v], mesh.P[3 * v + 1], mesh.P[3 * v + 2]});
      }
      const size_t vbase = out.positions.size() / 3;
      for (int k = 0; k < 3; ++k) {
        out.positions.push_back(p[k].x);
        out.positions.push_back(p[k].y);
        out.positions.push_back(p[k].z);
        out.indices.push_back(uint32_t(vbase + size_t(k)));
      }
      for (int k = 0; k < 3; ++k) {
        Vec3f n;
        if (has_n) {
          const size_t v = size_t(idx[k]);
          n = normalize3(xf_dir(xf, {mesh.N[3 * v], mesh.N[3 * v + 1], mesh.N[3 * v + 2]}));
        } else {
          n = normalize3(cross3(sub(p[1], p[0]), sub(p[2], p[0])));
        }
        out.normals.push_back(n.x);
        out.normals.push_back(n.y);
        out.normals.push_back(n.z);
        if (has_uv) {
          out.texcoords[2 * (vbase + size_t(k))] = mesh.uv[2 * size_t(idx[k])];
          out.texcoords[2 * (vbase + size_t(k)) + 1] = mesh.uv[2 * size_t(idx[k]) + 1];
        }
      }
      out.material_ids.push_back(mid);
      emissive += mesh.emissive ? 1u : 0u;
    }
  }

  phc_scene_desc &d = out.desc;
  d = phc_scene_desc{};
  d.positions = out.positions.data();
  d.vertex_count = out.positions.size() / 3;
  d.normals = out.normals.empty() ? nullptr : out.normals.data();
  d.indices = out.indices.data();
  d.triangle_count = out.indices.size() / 3;
  d.material_ids = out.material_ids.data();
  d.material_id_count = out.material_ids.size();
  d.material_count = uint32_t(out.materials.size());
  out.pt.materials = out.materials.data();
  out.pt.texcoords = out.texcoords.empty() ? nullptr : out.texcoords.data();
  out.pt.textures = out.textures.empty() ? nullptr : out.textures.data();
  out.pt.texture_count = uint32_t(out.textures.size());

  // environment image scaled, with the light's transform as its rotation
  // (pbrt_to_photon.cpp:432-467)
  bool env_loaded = false;
  if (ps.has_env && !ps.env_file.empty()) {
    Image env;
    if (load_image(base + ps.env_file, env)) {
      env_loaded = true;
      out.env_pixels.resize(env.rgb.size());
      for (size_t i = 0; i < env.rgb.size(); ++i)
        out.env_pixels[i] = env.rgb[i] * ps.env_scale;
      const Mat4 xf = from_column_major(ps.env_xf);
      const Mat4 inv = inverse(xf);
      phc_environment &e = d.environment;
      e.present = 1;
      e.visible = 1;
      e.width = uint32_t(env.width);
      e.height = uint32_t(env.height);
      e.pixels = out.env_pixels.data();
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          e.world_to_map[r * 3 + c] = inv.m[r][c];
          out.pt.env_map_to_world[r * 3 + c] = xf.m[r][c];
        }
      out.pt.env_map_to_world_given = 1;
    }
  }
  // instanced geometry (pbrt_to_photon.cpp:470-503): each object's
  // sub-meshes merged in object space (their own transforms unused), normals
  // only when every sub-mesh has them, the last sub-mesh's material; one
  // placement per ObjectInstance.  Only with use_instancing: otherwise the
  // instances are flattened into the mesh above, as the reference's
  // single-level back-end renders them.
  if (use_instancing && !ps.objects.empty() && !ps.instances.empty()) {
    std::map<std::string, uint32_t> obj_id;
    for (const auto &kv : ps.objects) {
      obj_id[kv.first] = uint32_t(out.object_data.size());
      phc_pbrt_scene::ObjectData od;
      uint32_t mid = 0, voff = 0;
      size_t nsum = 0, psum = 0;
      for (const Mesh &m : kv.second) {
        const auto it = mat_id.find(m.material);
        mid = it != mat_id.end() ? it->second : 0u;
        od.positions.insert(od.positions.end(), m.P.begin(), m.P.end());
        for (int v : m.indices) {
          if (v < 0 || size_t(v) >= m.P.size() / 3)
            throw std::out_of_range("pbrt: vertex index out of range in an object");
          od.indices.push_back(uint32_t(v) + voff);
        }
        if (m.N.size() >= m.P.size())
          od.normals.insert(od.normals.end(), m.N.begin(), m.N.begin() + std::ptrdiff_t(m.P.size()));
        nsum += m.N.size() >= m.P.size() ? m.P.size() : 0;
        psum += m.P.size();
        voff += uint32_t(m.P.size() / 3);
      }
      if (nsum < psum)
        od.normals.clear();
      out.object_data.push_back(std::move(od));
      phc_object ob{};
      ob.material_id = mid;
      out.objects.push_back(ob);
    }
    for (size_t o = 0; o < out.objects.size(); ++o) {
      const auto &od = out.object_data[o];
      phc_object &ob = out.objects[o];
      ob.positions = od.positions.data();
      ob.vertex_count = od.positions.size() / 3;
      ob.indices = od.indices.data();
      ob.triangle_count = od.indices.size() / 3;
      ob.normals = od.normals.empty() ? nullptr : od.normals.data();
    }
    for (const auto &pl : ps.instances) {
      const auto it = obj_id.find(pl.object);
      if (it == obj_id.end())
        continue;
      phc_instance in{};
      in.object_id = it->second;
      std::memcpy(in.transform, pl.xf, sizeof(in.transform));
      out.instances.push_back(in);
    }
    out.pt.objects = out.objects.data();
    out.pt.object_count = uint32_t(out.objects.size());
    out.pt.instances = out.instances.data();
    out.pt.instance_count = uint32_t(out.instances.size());
  }
  d.pt = &out.pt;

  // camera: LookAt, else the inverse of the camera transform
  // (pbrt_to_photon.cpp:468-488)
  Vec3f pos, dir, up;
  if (ps.cam.lookat) {
    pos = ps.cam.from;
    dir = normalize3(sub(ps.cam.at, pos));
    up = normalize3(ps.cam.up);
  } else {
    const Mat4 c2w = inverse(from_column_major(ps.cam.xf));
    pos = xf_point(c2w, {0.f, 0.f, 0.f});
    dir = normalize3(xf_dir(c2w, {0.f, 0.f, 1.f}));
    up = normalize3(xf_dir(c2w, {0.f, 1.f, 0.f}));
  }
  phc_camera &c = out.camera;
  phc_camera_default(&c);
  set3(c.position, pos.x, pos.y, pos.z);
  set3(c.direction, dir.x, dir.y, dir.z);
  set3(c.up, up.x, up.y, up.z);
  c.orthographic = 0;
  c.fovy = fovy_for_degrees(ps.cam.fov);
  c.aspect = float(ps.width) / float(ps.height);
  // make_perspective keeps the image plane at distance 1; a lens only adds
  // the aperture (the reference sets focus_dist afterwards, which ray
  // generation does not read)
  c.aperture_radius = ps.cam.lensradius > 0.f ? ps.cam.lensradius : 0.f;
  c.focus_distance = 1.f;

  // PathTracer::params defaults with the file's size, spp and depth
  phc_settings &s = out.settings;
  phc_settings_default(&s);
  s.width = uint32_t(std::max(ps.width, 1));
  s.height = uint32_t(std::max(ps.height, 1));
  s.pixel_samples = uint32_t(std::max(ps.spp, 1));
  s.max_depth = uint32_t(std::max(ps.max_depth, 0));
  s.background[0] = s.background[1] = s.background[2] = 0.f;
  s.background[3] = 1.f;
  s.ambient_color[0] = s.ambient_color[1] = s.ambient_color[2] = 1.f;
  s.ambient_radiance = 0.f;
  s.adaptive_sampling = 1;
  s.throughput_clamp = 10.f;
  s.max_diffuse_bounces = s.max_glossy_bounces = s.max_transmission_bounces = s.max_volume_bounces = -1;
  s.clamp_direct = s.clamp_indirect = 0.f;

  phc_pbrt_info &in = out.info;
  in.meshes = ps.meshes.size();
  in.named_materials = ps.materials.size();
  in.textures = ps.textures.size();
  in.loaded_textures = out.textures.size();
  in.object_defs = ps.objects.size();
  in.object_instances = ps.instances.size();
  in.triangles = d.triangle_count;
  in.emissive_triangles = emissive;
  in.width = s.width;
  in.height = s.height;
  in.spp = s.pixel_samples;
  in.max_depth = s.max_depth;
  in.has_env_map = env_loaded ? 1 : 0;
}

int fail(int code, const std::string &msg)
{
  phc::set_global_error(msg);
  return code;
}

} // namespace

extern "C" {

int phc_pbrt_load(const char *path, const phc_pbrt_options *options, phc_pbrt_scene **out)
{
  if (!out)
    return fail(PHC_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (!path)
    return fail(PHC_ERR_INVALID, "null path");
  try {
    {
      std::ifstream probe(path);
      if (!probe.is_open())
        return fail(PHC_ERR_INVALID, std::string("cannot open ") + path);
    }
    const bool instancing = options && options->use_instancing != 0;
    Parsed ps = parse(path, instancing);
    if (options) { // command-line overrides (photon_pbrt_render.cpp:120-123)
      if (options->width > 0)
        ps.width = options->width;
      if (options->height > 0)
        ps.height = options->height;
      if (options->spp > 0)
        ps.spp = options->spp;
      if (options->max_depth > 0)
        ps.max_depth = options->max_depth;
    }
    auto sc = std::make_unique<phc_pbrt_scene>();
    convert(ps, dir_of(path), instancing, *sc);
    *out = sc.release();
    return PHC_OK;
  } catch (const std::bad_alloc &) {
    return fail(PHC_ERR_OOM, "host allocation failed");
  } catch (const std::length_error &e) {
    return fail(PHC_ERR_LIMIT, e.what());
  } catch (const std::exception &e) {
    return fail(PHC_ERR_INVALID, e.what());
  }
}

void phc_pbrt_free(phc_pbrt_scene *scene) { delete scene; }

int phc_pbrt_scene_desc(const phc_pbrt_scene *scene, const phc_scene_desc **desc)
{
  if (!scene || !desc)
    return fail(PHC_ERR_INVALID, "null argument");
  *desc = &scene->desc;
  return PHC_OK;
}

int phc_pbrt_camera(const phc_pbrt_scene *scene, phc_camera *camera)
{
  if (!scene || !camera)
    return fail(PHC_ERR_INVALID, "null argument");
  *camera = scene->camera;
  return PHC_OK;
}

int phc_pbrt_settings(const phc_pbrt_scene *scene, phc_settings *settings)
{
  if (!scene || !settings)
    return fail(PHC_ERR_INVALID, "null argument");
  *settings = scene->settings;
  return PHC_OK;
}

int phc_pbrt_info_get(const phc_pbrt_scene *scene, phc_pbrt_info *info)
{
  if (!scene || !info)
    return fail(PHC_ERR_INVALID, "null argument");
  *info = scene->info;
  return PHC_OK;
}

} // extern "C"
