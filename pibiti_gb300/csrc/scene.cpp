// scene.cpp -- Scenes.xml loading and the scene's derived constants, on the
// host (the replacement for Scene, source/SPH/Scene*.cpp, and for
// cSPH::LoadScenes / cSPH::Reset).
//
// The XML reader is a small one of this library's own: elements, attributes
// in single or double quotes, comments, declarations and text (ignored).
// The scene semantics follow the reference exactly, because they decide the
// bytes of SimParams: the same defaults (Scene.cpp:7-66), the attributes in
// the same order with the same parsers (atof, strtol base 0, "%f %f %f";
// Scene_Load.cpp:11-111, header.h toFloat/toInt/toVec3), and the same
// derivations with the same float/double evaluation (Scene.cpp:69-113:
// pow(float, int) is evaluated in double, pow(float, float) in float).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "pibiti_sph.h"
#include "sph_internal.h"

namespace sph {
namespace {

// ---- minimal XML --------------------------------------------------------
struct XmlElem {
  std::string name;
  std::vector<std::pair<std::string, std::string>> attrs;
  std::vector<std::unique_ptr<XmlElem>> kids;
  const char* attr(const char* k) const {
    for (const auto& a : attrs)
      if (a.first == k) return a.second.c_str();
    return nullptr;
  }
};

class XmlReader {
 public:
  explicit XmlReader(const std::string& text) : s_(text), i_(0) {}

  // Parses the whole document; returns the root element or null.
  std::unique_ptr<XmlElem> parse(std::string* err) {
    std::unique_ptr<XmlElem> root;
    while (skip_misc()) {
      if (root) {  // a second top-level element: keep the first like TinyXML
        auto extra = element(err);
        if (!extra) return nullptr;
        continue;
      }
      root = element(err);
      if (!root) return nullptr;
    }
    if (!root) *err = "no root element";
    return root;
  }

 private:
  const std::string& s_;
  size_t i_;

  bool eof() const { return i_ >= s_.size(); }
  void ws() {
    while (!eof() && isspace((unsigned char)s_[i_])) ++i_;
  }
  bool starts(const char* p) const { return s_.compare(i_, strlen(p), p) == 0; }
  // Skips whitespace, comments, declarations and text; true at a '<' of an
  // element start.
  bool skip_misc() {
    for (;;) {
      while (!eof() && s_[i_] != '<') ++i_;
      if (eof()) return false;
      if (starts("<!--")) {
        size_t e = s_.find("-->", i_ + 4);
        i_ = e == std::string::npos ? s_.size() : e + 3;
      } else if (starts("<?")) {
        size_t e = s_.find("?>", i_ + 2);
        i_ = e == std::string::npos ? s_.size() : e + 2;
      } else if (starts("<!")) {
        size_t e = s_.find('>', i_ + 2);
        i_ = e == std::string::npos ? s_.size() : e + 1;
      } else if (starts("</")) {
        return true;  // caller handles end tags
      } else {
        return true;
      }
    }
  }
  std::string name() {
    size_t b = i_;
    while (!eof() && !isspace((unsigned char)s_[i_]) && s_[i_] != '>' && s_[i_] != '/' &&
           s_[i_] != '=')
      ++i_;
    return s_.substr(b, i_ - b);
  }
  static std::string unescape(const std::string& v) {
    std::string o;
    for (size_t k = 0; k < v.size(); ++k) {
      if (v[k] == '&') {
        static const char* ent[][2] = {{"&lt;", "<"}, {"&gt;", ">"}, {"&amp;", "&"},
                                       {"&quot;", "\""}, {"&apos;", "'"}};
        bool hit = false;
        for (auto& e : ent)
          if (v.compare(k, strlen(e[0]), e[0]) == 0) {
            o += e[1];
            k += strlen(e[0]) - 1;
            hit = true;
            break;
          }
        if (!hit) o += v[k];
      } else {
        o += v[k];
      }
    }
    return o;
  }
  std::unique_ptr<XmlElem> element(std::string* err) {
    if (eof() || s_[i_] != '<' || starts("</")) {
      *err = "expected an element";
      return nullptr;
    }
    ++i_;
    auto e = std::make_unique<XmlElem>();
    e->name = name();
    if (e->name.empty()) {
      *err = "empty element name";
      return nullptr;
    }
    for (;;) {
      ws();
      if (eof()) {
        *err = "unterminated start tag <" + e->name;
        return nullptr;
      }
      if (starts("/>")) {
        i_ += 2;
        return e;
      }
      if (s_[i_] == '>') {
        ++i_;
        break;
      }
      std::string k = name();
      if (k.empty()) {
        *err = "bad attribute in <" + e->name;
        return nullptr;
      }
      ws();
      if (eof() || s_[i_] != '=') {
        *err = "attribute " + k + " has no value";
        return nullptr;
      }
      ++i_;
      ws();
      if (eof() || (s_[i_] != '"' && s_[i_] != '\'')) {
        *err = "attribute " + k + " is not quoted";
        return nullptr;
      }
      const char q = s_[i_++];
      size_t b = i_;
      while (!eof() && s_[i_] != q) ++i_;
      if (eof()) {
        *err = "unterminated attribute " + k;
        return nullptr;
      }
      e->attrs.emplace_back(k, unescape(s_.substr(b, i_ - b)));
      ++i_;
    }
    // children until the matching end tag
    for (;;) {
      if (!skip_misc()) {
        *err = "missing </" + e->name + ">";
        return nullptr;
      }
      if (starts("</")) {
        i_ += 2;
        std::string n = name();
        ws();
        if (n != e->name || eof() || s_[i_] != '>') {
          *err = "mismatched end tag </" + n + "> for <" + e->name + ">";
          return nullptr;
        }
        ++i_;
        return e;
      }
      auto k = element(err);
      if (!k) return nullptr;
      e->kids.push_back(std::move(k));
    }
  }
};

int read_file(const char* path, std::string* out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail(SPH_ERR_XML, "cannot open %s", path);
  std::stringstream ss;
  ss << f.rdbuf();
  *out = ss.str();
  return SPH_OK;
}

int parse_doc(const std::string& text, std::unique_ptr<XmlElem>* root) {
  std::string err;
  XmlReader r(text);
  *root = r.parse(&err);
  if (!*root) return fail(SPH_ERR_XML, "XML: %s", err.c_str());
  return SPH_OK;
}

std::vector<const XmlElem*> scenes_of(const XmlElem& root) {
  std::vector<const XmlElem*> v;
  for (const auto& k : root.kids)
    if (k->name == "Scene") v.push_back(k.get());
  return v;
}

// ---- Scene semantics ------------------------------------------------------
const float kPi = 3.141592654f;  // Params.cuh:18

sph_float3 f3(float x, float y, float z) {
  sph_float3 v;
  v.x = x;
  v.y = y;
  v.z = z;
  return v;
}
sph_float3 operator+(sph_float3 a, sph_float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
sph_float3 operator-(sph_float3 a, sph_float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
sph_float3 operator*(sph_float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }

// header.h:144-156
float to_float(const char* s) { return (float)atof(s); }
int to_int(const char* s) { return (int)strtol(s, nullptr, 0); }
sph_float3 to_vec3(const char* s) {
  sph_float3 v = f3(0.f, 0.f, 0.f);
  sscanf(s, "%f %f %f", &v.x, &v.y, &v.z);
  return v;
}

struct SceneState {
  SimParams p;
  SphSceneInfo info;
  float rVel, r2Vel;
  SphEmitter emit[SPH_NUM_EMIT];
};

// Scene::InitDefault (Scene.cpp:7-66)
void init_default(SceneState& s) {
  memset(&s, 0, sizeof(s));
  SimParams& p = s.p;
  p.numParticles = 7 * 8 * 1024;
  p.maxParInCell = 16;
  p.timeStep = 0.0026f;
  p.globalDamping = 1.00f;
  p.gravity = f3(0, (float)-9.81, 0);
  p.particleR = (float)0.004;
  p.minDist = (float)1.0;
  p.h = (float)0.01;
  s.info.spacing = (float)1.38;
  p.restDensity = 1000;
  p.minDens = (float)1.0;
  p.stiffness = (float)3.0;
  p.viscosity = (float)0.5;
  const sph_float3 w = f3((float)0.2, (float)0.25, (float)0.2);
  p.worldMin = f3(-w.x, -w.y, -w.z);
  p.worldMax = w;
  s.info.initMin = p.worldMin;
  s.info.initMax = w;
  s.info.cellSize = (float)(p.particleR * 2.0);
  s.info.dropR = 5;
  s.info.rain = 0;
  s.info.initType = 0;
  s.info.initLast = 1;
  p.distBndSoft = 8;
  p.distBndHard = 1;
  p.bndStiff = 30000;
  p.bndDamp = 256;
  p.bndDampC = 60;
  p.bndType = SPH_BND_BOX;
  p.bndEffZ = SPH_BND_EFF_NONE;
  p.iHmap = 0;
  p.collR = (float)0.05;
  p.collPos.x = -77.f;
  p.spring = 80;
  p.damping = (float)0.02;
  p.shear = (float)0.1;
  p.angOut = (float)0.7;
  p.hClose = (float)-0.03;
  p.radIn = (float)0.4;
  p.s1 = (float)0.90;
  p.s2 = (float)0.90;
  p.s3 = (float)1.198;
  p.s4 = (float)0.7782;
  p.s5 = (float)0.8696;
  p.s6 = (float)0.843;
  p.rVexit = (float)0.03;
  p.rDexit = (float)0.04;
  p.rotType = 0;
  p.rAngle = 0;
  p.rotBlades = 4;
  p.rTwist = (float)0.04;
  p.rotSize.x = 0;
  p.rotSize.y = 4;
  p.rotSize.z = 12;
  p.rotR = 3;
  p.rotSpc = (float)0.7;
  p.r2Dist = 0;
  p.r2Angle = 0;
  p.r2twist = 1;
  s.rVel = 0;
  s.r2Vel = 1;
  for (SphEmitter& em : s.emit) em.vel = 1.5f;  // Emitter() (Scene.h:13)
  snprintf(s.info.title, sizeof(s.info.title), "No name");
  s.info.chapter = 0;
  for (int i = 0; i < SPH_NUM_ACC; ++i) {
    p.acc[i].pos = f3(0, 0, 0);
    p.acc[i].size = f3((float)0.005, (float)0.010, (float)0.005);
    p.acc[i].acc = f3(0, 10, 0);
    p.acc[i].type = SPH_ACC_OFF;
  }
  p.clrType = SPH_CLR_VELACC;
  p.brightness = (float)0.3;
  p.contrast = (float)0.3;
  p.iHue = 0;
  p.dyeType = 0;
  p.dyeClear = 2;
  p.dyeFade = 1.f;
  p.dyePos = f3(0, (float)-0.21, 0);
  p.dyeSize = f3((float)0.008, (float)0.012, (float)0.008);
}

// Scene::_FromXML (Scene_Load.cpp:11-111), attribute for attribute in the
// same order, so later attributes override earlier ones the same way.
void from_xml(SceneState& s, const XmlElem& e) {
  SimParams& p = s.p;
  SphSceneInfo& in = s.info;
  const char* a;
#define A(k) if ((a = e.attr(k)))
#define AF(k, v) A(k) { v = to_float(a); }
#define AI(k, v) A(k) { v = to_int(a); }
#define AV(k, v) A(k) { v = to_vec3(a); }
  A("World") {
    const sph_float3 w = to_vec3(a);
    p.worldMin = w * -0.5f;
    p.worldMax = w * 0.5f;
    in.initMin = w * -0.5f;
    in.initMax = w * 0.5f;
  }
  A("Init") {
    const sph_float3 w = to_vec3(a);
    in.initMin = w * -0.5f;
    in.initMax = w * 0.5f;
  }
  AV("WorldMin", p.worldMin);
  AV("InitMin", in.initMin);
  AV("WorldMax", p.worldMax);
  AV("InitMax", in.initMax);
  AI("InitType", in.initType);
  AI("InitLast", in.initLast);
  AF("CellSize", in.cellSize);
  A("name") snprintf(in.title, sizeof(in.title), "%s", a);
  A("chapter") in.chapter = 1;
  AF("dropR", in.dropR);
  AI("rain", in.rain);
  // emitters (Scene_Load.cpp:44-54): the first in attributes, up to
  // SPH_NUM_EMIT as <Emitter> children (which start again at index 0)
  AI("EmitSize", s.emit[0].size);
  AV("EmitPos", s.emit[0].pos);
  AF("EmitVel", s.emit[0].vel);
  AI("EmitSize2", s.emit[0].size2);
  AV("EmitRot", s.emit[0].rot);
  {
    int ie = 0;
    for (const auto& k : e.kids) {
      if (k->name != "Emitter" || ie >= SPH_NUM_EMIT) continue;
      SphEmitter& em = s.emit[ie++];
      if ((a = k->attr("size"))) em.size = to_int(a);
      if ((a = k->attr("pos"))) em.pos = to_vec3(a);
      if ((a = k->attr("vel"))) em.vel = to_float(a);
      if ((a = k->attr("size2"))) em.size2 = to_int(a);
      if ((a = k->attr("rot"))) em.rot = to_vec3(a);
    }
  }
  // accelerators as children (max NumAcc)
  int i = 0;
  for (const auto& k : e.kids) {
    if (k->name != "Accel" || i >= SPH_NUM_ACC) continue;
    if ((a = k->attr("type"))) p.acc[i].type = (uint32_t)to_int(a);
    if ((a = k->attr("pos"))) p.acc[i].pos = to_vec3(a);
    if ((a = k->attr("size"))) p.acc[i].size = to_vec3(a);
    if ((a = k->attr("acc"))) p.acc[i].acc = to_vec3(a);
    ++i;
  }
  AF("ColliderR", p.collR);
  A("ColliderPos") {
    const sph_float3 v = to_vec3(a);
    p.collPos.x = v.x;
    p.collPos.y = v.y;
    p.collPos.z = v.z;
    p.collPos.w = 1;
  }
  AF("spring", p.spring);
  AF("damping", p.damping);
  AF("shear", p.shear);
  A("Particles") p.numParticles = (uint32_t)to_int(a);
  A("ParticlesK") p.numParticles = (uint32_t)(to_int(a) * 1024);
  A("maxParInCell") p.maxParInCell = (uint32_t)to_int(a);
  AF("TimeStep", p.timeStep);
  AF("globalDamping", p.globalDamping);
  AV("Gravity", p.gravity);
  AF("particleR", p.particleR);
  AF("minDist", p.minDist);
  AF("particleH", p.h);
  AF("spacing", in.spacing);
  AF("RestDensity", p.restDensity);
  AF("minDens", p.minDens);
  AF("Stiffness", p.stiffness);
  AF("Viscosity", p.viscosity);
  AF("distBndSoft", p.distBndSoft);
  AF("bndStiff", p.bndStiff);
  AF("distBndHard", p.distBndHard);
  AF("bndDamp", p.bndDamp);
  AF("bndDampC", p.bndDampC);
  A("bndType") p.bndType = (uint32_t)to_int(a);
  A("bndEffZ") p.bndEffZ = (uint32_t)to_int(a);
  AI("HmapType", p.iHmap);
  AF("PumpAngOut", p.angOut);
  AF("PumpHClose", p.hClose);
  AF("PumpRadIn", p.radIn);
  AF("ExitVel", p.rVexit);
  AF("ExitDist", p.rDexit);
  AF("s1", p.s1);
  AF("s2", p.s2);
  AF("s3", p.s3);
  AF("s4", p.s4);
  AF("s5", p.s5);
  AF("s6", p.s6);
  A("RotorSizes") {
    const sph_float3 v = to_vec3(a);
    p.rotSize.x = (int)v.x;
    p.rotSize.y = (int)v.y;
    p.rotSize.z = (int)v.z;
  }
  AI("RotorType", p.rotType);
  AF("Rotor2Dist", p.r2Dist);
  AF("RotorVel", s.rVel);
  AF("Rotor2Vel", s.r2Vel);
  A("RotorAngle") p.rAngle = to_float(a) * kPi / 180.f;
  A("Rotor2Angle") p.r2Angle = to_float(a) * kPi / 180.f;
  AF("colParR", p.rotR);
  AF("colParSpc", p.rotSpc);
  AI("RotorBlades", p.rotBlades);
  AF("RotorTwist", p.rTwist);
  A("WaveSpeed") {
    s.rVel = to_float(a);
    p.rAngle = -kPi / 2.f;
  }
  AF("WaveAmpl", p.rTwist);
  AF("HSlope", p.r2Angle);
  AF("Hheight", p.r2Angle);
  AF("Hscale", p.hClose);
  AF("HxFq", p.s1);
  AF("HxOfs", p.s2);
  AF("HzFq", p.s3);
  AF("HzOfs", p.s4);
  AF("HholeR", p.s5);
  in.is_default = (e.attr("default") || e.attr("def")) ? 1 : 0;
#undef A
#undef AF
#undef AI
#undef AV
}

// Scene::_UpdatePar and Scene::_UpdateGrid (Scene.cpp:76-113).
void update(SceneState& s) {
  SimParams& p = s.p;
  SphSceneInfo& in = s.info;
  p.minDist *= p.particleR;
  p.h2 = p.h * p.h;
  in.spacing *= p.particleR;
  p.Poly6Kern = (float)(315.0f / ((double)(64.0f * kPi) * std::pow((double)p.h, 9.0)));
  p.SpikyKern = (float)((-0.5f * -45.0f) / ((double)kPi * std::pow((double)p.h, 6.0)));
  p.LapKern = (float)(45.0f / ((double)kPi * std::pow((double)p.h, 6.0)));
  p.minDens = 1.f / powf(p.minDens * p.restDensity, 2.f);
  p.particleMass = p.restDensity * 4.f / 3.f * kPi * powf(p.particleR, 3.f);
  p.distBndSoft *= p.particleR;
  p.distBndHard *= p.particleR;
  p.rotR *= p.particleR;
  p.rotSpc *= p.rotR;

  const float b = p.distBndSoft - p.particleR;
  const sph_float3 b3 = f3(b, b, b);
  p.worldMinD = p.worldMin + b3;
  p.worldMaxD = p.worldMax - b3;
  in.initMin = in.initMin + b3;
  in.initMax = in.initMax - b3;
  p.worldSize = p.worldMax - p.worldMin;
  p.worldSizeD = p.worldMaxD - p.worldMinD;
  p.cellSize = f3(in.cellSize, in.cellSize, in.cellSize);
  p.gridSize.x = (uint32_t)std::ceil(p.worldSize.x / p.cellSize.x);
  p.gridSize.y = (uint32_t)std::ceil(p.worldSize.y / p.cellSize.y);
  p.gridSize.z = (uint32_t)std::ceil(p.worldSize.z / p.cellSize.z);
  p.gridSize_yx = p.gridSize.y * p.gridSize.x;
  p.numCells = p.gridSize.x * p.gridSize.y * p.gridSize.z;
  if (p.collPos.x == -77.f) {
    p.collPos.x = p.worldMin.x + b - p.collR * 1.2f;
    p.collPos.y = p.worldMin.y + b + p.collR * 1.f;
    p.collPos.z = 0;
    p.collPos.w = 1;
  }
}

void finish(const SceneState& s, SimParams* out, SphSceneInfo* info) {
  *out = s.p;
  if (info) *info = s.info;
}

void motion_of(const SceneState& s, SphSceneMotion* m) {
  memset(m, 0, sizeof(*m));
  for (int k = 0; k < SPH_NUM_EMIT; ++k) m->emit[k] = s.emit[k];
  m->rVel = s.rVel;
  m->r2Vel = s.r2Vel;
}

int scene_element(const std::string& xml, std::unique_ptr<XmlElem>* root, const XmlElem** e) {
  SPH_TRY(parse_doc(xml, root));
  *e = root->get();
  if ((*e)->name != "Scene") {
    const auto sc = scenes_of(**root);
    if (sc.empty()) return fail(SPH_ERR_XML, "no <Scene> element");
    *e = sc[0];
  }
  return SPH_OK;
}

// rand()/RAND_MAX stand-in for cSPH::Reset's random fill: splitmix64.
struct Rng {
  uint64_t x;
  float next() {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)((z >> 40) * (1.0 / 16777216.0));
  }
};

}  // namespace
}  // namespace sph

using namespace sph;

extern "C" {

int sph_scene_count(const char* path, int* count) {
  if (!path || !count) return fail(SPH_ERR_ARG, "scene_count: null argument");
  std::string text;
  SPH_TRY(read_file(path, &text));
  std::unique_ptr<XmlElem> root;
  SPH_TRY(parse_doc(text, &root));
  *count = (int)scenes_of(*root).size();
  return SPH_OK;
}

int sph_scene_load(const char* path, int index, SimParams* out, SphSceneInfo* info) {
  if (!path || !out) return fail(SPH_ERR_ARG, "scene_load: null argument");
  std::string text;
  SPH_TRY(read_file(path, &text));
  std::unique_ptr<XmlElem> root;
  SPH_TRY(parse_doc(text, &root));
  const auto sc = scenes_of(*root);
  if (index < 0 || index >= (int)sc.size())
    return fail(SPH_ERR_ARG, "scene index %d out of range (%zu scenes)", index, sc.size());
  SceneState s;
  init_default(s);
  from_xml(s, *sc[index]);
  update(s);
  finish(s, out, info);
  return SPH_OK;
}

int sph_scene_parse(const char* xml, SimParams* out, SphSceneInfo* info) {
  if (!xml || !out) return fail(SPH_ERR_ARG, "scene_parse: null argument");
  std::unique_ptr<XmlElem> root;
  SPH_TRY(parse_doc(std::string(xml), &root));
  const XmlElem* e = root.get();
  if (e->name != "Scene") {
    const auto sc = scenes_of(*root);
    if (sc.empty()) return fail(SPH_ERR_XML, "no <Scene> element");
    e = sc[0];
  }
  SceneState s;
  init_default(s);
  from_xml(s, *e);
  update(s);
  finish(s, out, info);
  return SPH_OK;
}

int sph_scene_default(SimParams* out, SphSceneInfo* info) {
  if (!out) return fail(SPH_ERR_ARG, "scene_default: null argument");
  SceneState s;
  init_default(s);
  update(s);
  finish(s, out, info);
  return SPH_OK;
}

int sph_scene_default_index(const char* path, int* index) {
  if (!path || !index) return fail(SPH_ERR_ARG, "scene_default_index: null argument");
  std::string text;
  SPH_TRY(read_file(path, &text));
  std::unique_ptr<XmlElem> root;
  SPH_TRY(parse_doc(text, &root));
  const auto sc = scenes_of(*root);
  *index = 0;
  for (size_t i = 0; i < sc.size(); ++i)
    if (sc[i]->attr("default") || sc[i]->attr("def")) *index = (int)i;
  return SPH_OK;
}

// cSPH::Reset (SPH_Init.cpp:23-79).
int sph_scene_reset(const SimParams* params, const SphSceneInfo* info, int type, uint64_t seed,
                    sph_float4* pos, sph_float4* vel, uint32_t* placed) {
  if (!params || !info || !pos || !vel) return fail(SPH_ERR_ARG, "scene_reset: null argument");
  const SimParams& p = *params;
  const uint32_t N = p.numParticles;
  const float r = p.particleR, spc = info->spacing, b = p.distBndSoft;
  const sph_float3 cp = f3(p.collPos.x, p.collPos.y, p.collPos.z);
  sph_float3 wMin = p.worldMinD, wSize = p.worldSizeD;
  sph_float3 imin = info->initMin, imax = info->initMax;
  imin.y += r;
  wMin.x += r;
  wMin.y += r;
  wMin.z += r;
  wSize.x -= 2 * r;
  wSize.y -= 2 * r;
  wSize.z -= 2 * r;
  uint32_t i = 0;
  auto put = [&](float x, float y, float z) {
    pos[i].x = x;
    pos[i].y = y;
    pos[i].z = z;
    pos[i].w = 1.f;
    vel[i].x = vel[i].y = vel[i].z = vel[i].w = 0.f;
    ++i;
  };
  if (type == 1) {
    Rng g{seed};
    while (i < N) {
      const float x = wMin.x + wSize.x * g.next();
      const float y = wMin.y + wSize.y * g.next();
      const float z = wMin.z + wSize.z * g.next();
      put(x, y, z);
    }
  } else {
    if (!(spc > 0.f)) return fail(SPH_ERR_PARAMS, "scene_reset: spacing must be positive");
    float px = imin.x, py = imin.y, pz = imin.z;
    // INC (SPH_Init.cpp:41-48): the first named axis runs fastest.
    auto inc = [&]() {
      float* ax[3];
      float lo[3], hi[3];
      const int last = info->initLast;
      const int order[3][3] = {{1, 2, 0}, {0, 2, 1}, {0, 1, 2}};  // 0: y,z,x  1: x,z,y  2: x,y,z
      const int* o = order[(last == 0 || last == 2) ? last : 1];
      float* P[3] = {&px, &py, &pz};
      const float L[3] = {imin.x, imin.y, imin.z}, H[3] = {imax.x, imax.y, imax.z};
      for (int k = 0; k < 3; ++k) {
        ax[k] = P[o[k]];
        lo[k] = L[o[k]];
        hi[k] = H[o[k]];
      }
      *ax[0] += spc;
      if (*ax[0] >= hi[0]) {
        *ax[0] = lo[0];
        *ax[1] += spc;
        if (*ax[1] >= hi[1]) {
          *ax[1] = lo[1];
          *ax[2] += spc;
          if (*ax[2] >= hi[2]) *ax[2] = lo[2];
        }
      }
    };
    // A volume that never accepts a position would loop forever in the
    // reference; stop after visiting far more lattice sites than exist.
    const double sites = std::ceil((double)(imax.x - imin.x) / spc + 1) *
                         std::ceil((double)(imax.y - imin.y) / spc + 1) *
                         std::ceil((double)(imax.z - imin.z) / spc + 1);
    const uint64_t limit = (uint64_t)N * 4 + (uint64_t)(sites > 0 ? sites : 0) * 2 + 1024;
    uint64_t visits = 0;
    if (p.bndType == SPH_BND_PUMP_Y) {
      const float rad = info->initMax.x, hc = p.hClose - b * 0.90f, rin = rad * p.radIn - b / 2;
      const float xs = sinf(p.angOut * p.s3) * rad - b / 2 - p.particleR;
      while (i < N && visits++ < limit) {
        if ((p.angOut < 0.5f && py > 0 && pz < hc && px < xs && px > -xs) ||
            (p.angOut >= 0.5f && py > 0 && pz < hc && px > 0.09f * p.s4) ||
            sqrtf(px * px + py * py) * 1.01f < (pz < hc ? rad : rin))
          put(px, py, pz);
        inc();
      }
    } else {
      while (i < N && visits++ < limit) {
        const float dx = px - cp.x, dy = py - cp.y, dz = pz - cp.z;
        if (sqrtf(dx * dx + dy * dy + dz * dz) > p.collR || p.rotType > 0) {
          if (p.bndType == SPH_BND_BOX || info->initType >= 9 || p.bndType == SPH_BND_CYL_YZ ||
              (p.bndType == SPH_BND_CYL_Y && sqrtf(px * px + pz * pz) < imax.x) ||
              (p.bndType == SPH_BND_CYL_Z && sqrtf(px * px + py * py) < -imin.y) ||
              (p.bndType == SPH_BND_SPHERE && sqrtf(px * px + py * py + pz * pz) < -imin.y))
            put(px, py, pz);
        }
        inc();
      }
    }
  }
  if (placed) *placed = i;
  if (i < N) return fail(SPH_ERR_PARAMS, "scene_reset: init volume accepted only %u of %u particles", i, N);
  return SPH_OK;
}

}  // extern "C"

extern "C" {

int sph_scene_load_motion(const char* path, int index, SphSceneMotion* out) {
  if (!path || !out) return fail(SPH_ERR_ARG, "scene_load_motion: null argument");
  std::string text;
  SPH_TRY(read_file(path, &text));
  std::unique_ptr<XmlElem> root;
  SPH_TRY(parse_doc(text, &root));
  const auto sc = scenes_of(*root);
  if (index < 0 || index >= (int)sc.size())
    return fail(SPH_ERR_ARG, "scene index %d out of range (%zu scenes)", index, sc.size());
  SceneState s;
  init_default(s);
  from_xml(s, *sc[index]);
  motion_of(s, out);
  return SPH_OK;
}

int sph_scene_parse_motion(const char* xml, SphSceneMotion* out) {
  if (!xml || !out) return fail(SPH_ERR_ARG, "scene_parse_motion: null argument");
  std::unique_ptr<XmlElem> root;
  const XmlElem* e = nullptr;
  SPH_TRY(scene_element(std::string(xml), &root, &e));
  SceneState s;
  init_default(s);
  from_xml(s, *e);
  motion_of(s, out);
  return SPH_OK;
}

// App::UpdateEmitter, emitter part (App/Update.cpp:64-91).  The rotation
// is the modelview matrix M = Rx(rot.x) Ry(-rot.y) (glRotatef in degrees)
// applied transposed (App::mulTr, Input.cpp:587-592): r = M^T v.
int sph_emitter_particles(const SphEmitter* em, float spacing, sph_float4* pos, sph_float4* vel,
                          uint32_t capacity, uint32_t* count) {
  if (!em || !count) return fail(SPH_ERR_ARG, "emitter_particles: null argument");
  *count = 0;
  if (em->size <= 0) return SPH_OK;
  const int ex = em->size, ey = em->size2 == 0 ? ex : em->size2;
  const uint32_t n = (uint32_t)ex * (uint32_t)ey;
  if (n > capacity || !pos || !vel) return fail(SPH_ERR_ARG, "emitter_particles: room for %u particles needed", n);
  const float deg = 3.14159265358979f / 180.f;
  const float ca = cosf(em->rot.x * deg), sa = sinf(em->rot.x * deg);
  const float cb = cosf(-em->rot.y * deg), sb = sinf(-em->rot.y * deg);
  // M = Rx(a) Ry(b), row-major m[r][c]
  const float m[3][3] = {{cb, 0.f, sb}, {sa * sb, ca, -sa * cb}, {-ca * sb, sa, ca * cb}};
  auto mul_tr = [&](float x, float y, float z, float* r) {
    for (int c = 0; c < 3; ++c) r[c] = x * m[0][c] + y * m[1][c] + z * m[2][c];
  };
  float v3[3];
  mul_tr(0.f, 0.f, em->vel, v3);
  const float zx = (float)(ex - 1) * 0.5f, zy = (float)(ey - 1) * 0.5f;
  uint32_t i = 0;
  for (int y = 0; y < ey; ++y)
    for (int x = 0; x < ex; ++x, ++i) {
      float r[3];
      mul_tr(((float)x - zx) * spacing, ((float)y - zy) * spacing, -spacing, r);
      pos[i] = {r[0] + em->pos.x, r[1] + em->pos.y, r[2] + em->pos.z, 0.f};
      vel[i] = {v3[0], v3[1], v3[2], 0.f};
    }
  *count = n;
  return SPH_OK;
}

// cSPH::Drop (SPH_Init.cpp:83-117): a ball of particles of radius dropR
// spacings, at the box centre, or (random) at a random place near the top;
// at most `capacity` particles (the reference stops at numParticles).
int sph_drop_particles(const SimParams* params, const SphSceneInfo* info, int random,
                       uint64_t seed, sph_float4* pos, sph_float4* vel, uint32_t capacity,
                       uint32_t* count) {
  if (!params || !info || !count) return fail(SPH_ERR_ARG, "drop_particles: null argument");
  const SimParams& p = *params;
  const float r = info->dropR, spc = info->spacing, r2 = r * r, db = (r + 1.f) * spc, d = 0.5f;
  sph_float3 c = f3(0.5f, 0.5f, 0.5f);
  if (random) {
    Rng g{seed};
    const uint32_t t = p.bndType;
    c.y = (t == SPH_BND_BOX || t == SPH_BND_CYL_Y) ? 1.0f : 0.75f;
    if (t == SPH_BND_BOX || t == SPH_BND_CYL_Z) {
      c.x = g.next();
      c.z = g.next();
    } else {
      const float rr = g.next(), k = g.next() * 2.f * 3.14159265358979f;
      c.x = d + d * cosf(k) * rr;
      c.z = d - d * sinf(k) * rr;
    }
  }
  const sph_float3 ws = p.worldSizeD;
  const sph_float3 posw = f3(p.worldMinD.x + db + c.x * (ws.x - 2.f * db),
                             p.worldMinD.y + db + c.y * (ws.y - 2.f * db),
                             p.worldMinD.z + db + c.z * (ws.z - 2.f * db));
  const int ir = (int)-r;  // the reference's int loop bound from -r
  uint32_t n = 0;
  for (int z = ir; z <= r; ++z)
    for (int y = ir; y <= r; ++y)
      for (int x = ir; x <= r; ++x)
        if ((float)(x * x + y * y + z * z) <= r2 && n < capacity) {  // "a < numParticles"
          if (!pos || !vel) return fail(SPH_ERR_ARG, "drop_particles: null output");
          pos[n] = {x * spc + posw.x, y * spc + posw.y, z * spc + posw.z, 1.f};
          vel[n] = {0.f, 0.f, 0.f, 0.f};
          ++n;
        }
  *count = n;
  return SPH_OK;
}

// The per-frame parameter updates of App::UpdateEmitter (App/Update.cpp:
// 14-23): rotor angles and the dye-clear countdown.
int sph_scene_advance(SimParams* p, const SphSceneMotion* m) {
  if (!p || !m) return fail(SPH_ERR_ARG, "scene_advance: null argument");
  if (m->rVel != 0.f) {
    p->rAngle += m->rVel * p->timeStep;
    if (p->r2Dist > 0.f) {
      p->r2Angle += m->rVel * m->r2Vel * p->timeStep;
      p->r2twist = m->r2Vel < 0.f ? -1.f : 1.f;
    }
  }
  if (p->dyeClear > 0) p->dyeClear--;
  return SPH_OK;
}

}  // extern "C"
