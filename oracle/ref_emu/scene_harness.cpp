/*
 * scene_harness.cpp -- TEST INFRASTRUCTURE ONLY (part of the oracle).
 *
 * Drives the reference's own scene loader (Scene.cpp, Scene_Load.cpp, TinyXML,
 * all compiled unmodified from the reference tree by build_ref.sh) the way
 * cSPH::LoadScenes does (SPH_Scenes.cpp:171-202): every <Scene> element under
 * the document root becomes `Scene(TiXmlElement*)`, which applies the
 * defaults, the XML attributes and the derived constants.  The resulting
 * SimParams bytes are the golden vectors for the product's scene loader.
 */
#include "header.h"
#include "Scene.h"

namespace {
TiXmlElement* nth_scene(TiXmlDocument& doc, int index) {
  TiXmlElement* root = doc.RootElement();
  if (!root) return nullptr;
  TiXmlElement* s = root->FirstChildElement("Scene");
  for (int i = 0; s && i < index; ++i) s = s->NextSiblingElement("Scene");
  return s;
}
}  // namespace

extern "C" {

int ref_scene_count(const char* path) {
  TiXmlDocument doc;
  if (!doc.LoadFile(path)) return -1;
  TiXmlElement* root = doc.RootElement();
  if (!root) return -1;
  int n = 0;
  for (TiXmlElement* s = root->FirstChildElement("Scene"); s; s = s->NextSiblingElement("Scene"))
    ++n;
  return n;
}

/* extra[0] fCellSize, [1..3] initMin, [4..6] initMax, [7] initType,
   [8] initLast, [9] spacing, [10] dropR, [11] rain, [12] bChapter */
int ref_scene_load(const char* path, int index, SimParams* out, float* extra) {
  TiXmlDocument doc;
  if (!doc.LoadFile(path)) return -1;
  TiXmlElement* s = nth_scene(doc, index);
  if (!s) return -2;
  Scene sc(s);
  memcpy(out, &sc.params, sizeof(SimParams));
  extra[0] = sc.fCellSize;
  extra[1] = sc.initMin.x;
  extra[2] = sc.initMin.y;
  extra[3] = sc.initMin.z;
  extra[4] = sc.initMax.x;
  extra[5] = sc.initMax.y;
  extra[6] = sc.initMax.z;
  extra[7] = (float)sc.initType;
  extra[8] = (float)sc.initLast;
  extra[9] = sc.spacing;
  extra[10] = sc.dropR;
  extra[11] = (float)sc.rain;
  extra[12] = sc.bChapter ? 1.f : 0.f;
  return 0;
}

/* Emitters and rotor speeds of scene `index`: per emitter pos[3], rot[3],
   vel, size, size2 (9 floats, NumEmit emitters), then rVel, r2Vel. */
int ref_scene_motion(const char* path, int index, float* out) {
  TiXmlDocument doc;
  if (!doc.LoadFile(path)) return -1;
  TiXmlElement* s = nth_scene(doc, index);
  if (!s) return -2;
  Scene sc(s);
  for (int e = 0; e < NumEmit; ++e) {
    const Emitter& em = sc.emit[e];
    float* o = out + 9 * e;
    o[0] = em.pos.x;
    o[1] = em.pos.y;
    o[2] = em.pos.z;
    o[3] = em.rot.x;
    o[4] = em.rot.y;
    o[5] = em.rot.z;
    o[6] = em.vel;
    o[7] = (float)em.size;
    o[8] = (float)em.size2;
  }
  out[9 * NumEmit] = sc.rVel;
  out[9 * NumEmit + 1] = sc.r2Vel;
  return 0;
}

/* Scene() (Scene.h:56): defaults plus derivations, no XML. */
int ref_scene_default(SimParams* out, float* extra) {
  Scene sc;
  memcpy(out, &sc.params, sizeof(SimParams));
  extra[0] = sc.fCellSize;
  extra[9] = sc.spacing;
  return 0;
}

}  // extern "C"
