// ORACLE / TEST INFRASTRUCTURE ONLY. Nothing in the product links this file.
//
// Host driver for the snow reference's compute shaders compiled as C++
// (oracle/ref_translate.py). It plays the part of the reference's host code:
//   * buffer set-up with the std140 layouts of
//       ParticleSystem::initSSBO   (src/snow/object/particlesystem.cpp:101-228)
//       Grid::initSSBO             (src/snow/object/grid.cpp:74-148)
//       CollisionObjects::initSSBO (src/snow/object/collisionObjects.cpp:25-66)
//     bound to the binding points of src/snow/utils/defines.hpp:30-48;
//   * the dispatch shapes of src/snow/simulation/computingTechnique/*.cpp
//     ((N/1024+1, 64, 1) for the particle x neighbour kernels, (G/1024+1,1,1)
//     for the grid kernels, (numColliders,1,1) for rigidAdvance);
//   * the order of ExplicitTimeUpdate::init / ::update
//     (src/snow/simulation/timeUpdate/explicittimeupdate.cpp:4-63).
// The grid kernels gReset and gForceCompute have no bounds check and run
// (G/1024+1)*1024 invocations; the grid buffers are padded to that length so
// the extra invocations touch padding, as on the reference's GPU.
#include <cstring>
#include <vector>

#include "glsl_compat.hpp"

using namespace glslc;

extern "C" {
void snowref_dispatch_gReset(const RefBindings*, const RefUniforms*, unsigned, unsigned, unsigned, int);
void snowref_dispatch_rigidAdvance(const RefBindings*, const RefUniforms*, unsigned, unsigned, unsigned, int);
void snowref_dispatch_gMassCompute(const RefBindings*, const RefUniforms*, unsigned, unsigned, unsigned, int);
void snowref_dispatch_pVolumeCompute(const RefBindings*, const RefUniforms*, unsigned, unsigned, unsigned, int);
void snowref_dispatch_p2gTransfer(const RefBindings*, const RefUniforms*, unsigned, unsigned, unsigned, int);
void snowref_dispatch_gForceCompute(const RefBindings*, const RefUniforms*, unsigned, unsigned, unsigned, int);
void snowref_dispatch_g2pTransfer(const RefBindings*, const RefUniforms*, unsigned, unsigned, unsigned, int);
void snowref_dispatch_particleAdvance(const RefBindings*, const RefUniforms*, unsigned, unsigned, unsigned, int);
}

namespace {

// Binding points, src/snow/utils/defines.hpp:30-48.
enum {
  PARTICLE_POS_BUFFER = 0,
  PARTICLE_VEL_BUFFER = 1,
  GRID_POS_BUFFER = 2,
  GRID_VEL_BUFFER = 3,
  PARTICLE_FE_BUFFER = 4,
  PARTICLE_FP_BUFFER = 5,
  PARTICLE_VEL_N_BUFFER = 6,
  GRID_VEL_N_BUFFER = 7,
  COLLIDER_POS_BUFFER = 8,
  COLLIDER_VEL_BUFFER = 9,
  COLLIDER_NOR_BUFFER = 10,
  PARTICLE_DELTA_VEL_BUFFER_0 = 13,
  PARTICLE_DELTA_VEL_BUFFER_1 = 14,
  PARTICLE_DELTA_VEL_BUFFER_2 = 15,
  GRID_FORCE_BUFFER = 16,
};
constexpr unsigned kThreadsX = 1024;  // NUM_OF_GPGPU_THREADS_X
constexpr unsigned kNeighbours = 64;  // PARTICLE_TO_GRID_SIZE

}  // namespace

struct SnowRefDesc {
  float grid_pos[3];
  int grid_dim[3];
  float grid_spacing;
  float young, poisson, hardening, crit_compression, crit_stretch;
  int n_colliders;
  const float* collider_pos;       // n x 3
  const int* collider_type;        // n
  const float* collider_vel;       // n x 3
  const float* collider_radius;    // n
  const float* collider_normal;    // n x 3
  const float* collider_friction;  // n
  int threads;
};

struct SnowRef {
  RefUniforms u{};
  int threads = 1;
  unsigned N = 0;
  unsigned G = 0, Gpad = 0;
  unsigned ncoll = 0;
  std::vector<vec4> pxm, gxm, gvn, cx, cv, cn;
  std::vector<ivec4> pv, pvn, pd0, pd1, pd2, gv, gf;
  std::vector<mat4> pFE, pFP;
  RefBindings b{};

  void bind() {
    std::memset(&b, 0, sizeof(b));
    b.ptr[PARTICLE_POS_BUFFER] = pxm.data();
    b.ptr[PARTICLE_VEL_BUFFER] = pv.data();
    b.ptr[GRID_POS_BUFFER] = gxm.data();
    b.ptr[GRID_VEL_BUFFER] = gv.data();
    b.ptr[PARTICLE_FE_BUFFER] = pFE.data();
    b.ptr[PARTICLE_FP_BUFFER] = pFP.data();
    b.ptr[PARTICLE_VEL_N_BUFFER] = pvn.data();
    b.ptr[GRID_VEL_N_BUFFER] = gvn.data();
    b.ptr[COLLIDER_POS_BUFFER] = cx.data();
    b.ptr[COLLIDER_VEL_BUFFER] = cv.data();
    b.ptr[COLLIDER_NOR_BUFFER] = cn.data();
    b.ptr[PARTICLE_DELTA_VEL_BUFFER_0] = pd0.data();
    b.ptr[PARTICLE_DELTA_VEL_BUFFER_1] = pd1.data();
    b.ptr[PARTICLE_DELTA_VEL_BUFFER_2] = pd2.data();
    b.ptr[GRID_FORCE_BUFFER] = gf.data();
  }
};

extern "C" {

SnowRef* snowref_create(const SnowRefDesc* d) {
  SnowRef* s = new SnowRef();
  for (int i = 0; i < 3; i++) {
    s->u.gGridPos[i] = d->grid_pos[i];
    s->u.gGridDim[i] = d->grid_dim[i];
  }
  s->u.gridSpacing = d->grid_spacing;
  s->u.young = d->young;
  s->u.poisson = d->poisson;
  s->u.hardening = d->hardening;
  s->u.critComp = d->crit_compression;
  s->u.critStretch = d->crit_stretch;
  s->threads = d->threads;
  s->G = (unsigned)d->grid_dim[0] * (unsigned)d->grid_dim[1] * (unsigned)d->grid_dim[2];
  s->Gpad = (s->G / kThreadsX + 1) * kThreadsX;
  s->gxm.assign(s->Gpad, vec4(0.0f));
  s->gvn.assign(s->Gpad, vec4(0.0f));
  s->gv.assign(s->Gpad, ivec4(0, 0, 0, 0));
  s->gf.assign(s->Gpad, ivec4(0, 0, 0, 0));
  // Grid::initSSBO: node positions x_off + h * (float)i, i fastest (grid.cpp:96-107).
  const float h = d->grid_spacing;
  unsigned idx = 0;
  for (int k = 0; k < d->grid_dim[2]; k++)
    for (int j = 0; j < d->grid_dim[1]; j++)
      for (int i = 0; i < d->grid_dim[0]; i++)
        s->gxm[idx++] = vec4(d->grid_pos[0] + h * (float)i, d->grid_pos[1] + h * (float)j,
                             d->grid_pos[2] + h * (float)k, 0.0f);
  // CollisionObjects::initSSBO: cx = (pos, type), cv = (vel, radius), cn = (normal, friction).
  s->ncoll = (unsigned)d->n_colliders;
  for (int c = 0; c < d->n_colliders; c++) {
    s->cx.push_back(vec4(d->collider_pos[3 * c], d->collider_pos[3 * c + 1], d->collider_pos[3 * c + 2],
                         (float)d->collider_type[c]));
    s->cv.push_back(vec4(d->collider_vel[3 * c], d->collider_vel[3 * c + 1], d->collider_vel[3 * c + 2],
                         d->collider_radius[c]));
    s->cn.push_back(vec4(d->collider_normal[3 * c], d->collider_normal[3 * c + 1],
                         d->collider_normal[3 * c + 2], d->collider_friction[c]));
  }
  s->u.gNumColliders = s->ncoll;
  if (s->ncoll == 0) {  // keep the pointers valid
    s->cx.push_back(vec4(0.0f));
    s->cv.push_back(vec4(0.0f));
    s->cn.push_back(vec4(0.0f));
  }
  return s;
}

void snowref_destroy(SnowRef* s) { delete s; }

// std140 buffers exactly as ParticleSystem::initSSBO writes them:
// pxm N x vec4 (x, m); pv N x ivec4 (v * 1e8, volume slot); pFE, pFP N x mat4.
void snowref_upload(SnowRef* s, const float* pxm, const int* pv, const float* pFE, const float* pFP,
                    unsigned n) {
  s->N = n;
  s->u.indexSize = n;
  s->pxm.resize(n ? n : 1);
  s->pv.resize(n ? n : 1);
  s->pFE.resize(n ? n : 1);
  s->pFP.resize(n ? n : 1);
  if (n) {
    std::memcpy(s->pxm.data(), pxm, sizeof(vec4) * n);
    std::memcpy(s->pv.data(), pv, sizeof(ivec4) * n);
    std::memcpy(s->pFE.data(), pFE, sizeof(mat4) * n);
    std::memcpy(s->pFP.data(), pFP, sizeof(mat4) * n);
  }
  s->pvn.assign(n ? n : 1, ivec4(0, 0, 0, 0));
  s->pd0.assign(n ? n : 1, ivec4(0, 0, 0, 0));
  s->pd1.assign(n ? n : 1, ivec4(0, 0, 0, 0));
  s->pd2.assign(n ? n : 1, ivec4(0, 0, 0, 0));
  s->bind();
}

enum {
  SNOWREF_RIGID = 0,
  SNOWREF_RESET = 1,
  SNOWREF_P2G = 2,
  SNOWREF_GFORCE = 3,
  SNOWREF_G2P = 4,
  SNOWREF_ADVANCE = 5,
  SNOWREF_GMASS = 6,
  SNOWREF_PVOLUME = 7,
};

// One dispatch with the reference's shape (computingTechnique/*.cpp).
void snowref_dispatch(SnowRef* s, int which, double dt) {
  s->u.dt = (float)dt;  // glUniform1f of the double dt (technique.cpp:122-125)
  const unsigned pgroups = s->N / kThreadsX + 1;
  const unsigned ggroups = s->G / kThreadsX + 1;
  const RefBindings* b = &s->b;
  const RefUniforms* u = &s->u;
  switch (which) {
    case SNOWREF_RIGID: snowref_dispatch_rigidAdvance(b, u, s->ncoll, 1, 1, 1); break;
    case SNOWREF_RESET: snowref_dispatch_gReset(b, u, ggroups, 1, 1, s->threads); break;
    case SNOWREF_P2G: snowref_dispatch_p2gTransfer(b, u, pgroups, kNeighbours, 1, s->threads); break;
    case SNOWREF_GFORCE: snowref_dispatch_gForceCompute(b, u, ggroups, 1, 1, s->threads); break;
    case SNOWREF_G2P: snowref_dispatch_g2pTransfer(b, u, pgroups, kNeighbours, 1, s->threads); break;
    case SNOWREF_ADVANCE: snowref_dispatch_particleAdvance(b, u, pgroups, 1, 1, s->threads); break;
    case SNOWREF_GMASS: snowref_dispatch_gMassCompute(b, u, pgroups, kNeighbours, 1, s->threads); break;
    case SNOWREF_PVOLUME: snowref_dispatch_pVolumeCompute(b, u, pgroups, kNeighbours, 1, s->threads); break;
    default: break;
  }
}

// ExplicitTimeUpdate::init one-time passes (explicittimeupdate.cpp:29-33).
void snowref_init(SnowRef* s) {
  snowref_dispatch(s, SNOWREF_RESET, 0.0);
  snowref_dispatch(s, SNOWREF_GMASS, 0.0);
  snowref_dispatch(s, SNOWREF_PVOLUME, 0.0);
}

// ExplicitTimeUpdate::update (explicittimeupdate.cpp:36-63).
void snowref_update(SnowRef* s, double dt) {
  snowref_dispatch(s, SNOWREF_RIGID, dt);
  snowref_dispatch(s, SNOWREF_RESET, dt);
  snowref_dispatch(s, SNOWREF_P2G, dt);
  snowref_dispatch(s, SNOWREF_GFORCE, dt);
  snowref_dispatch(s, SNOWREF_G2P, dt);
  snowref_dispatch(s, SNOWREF_ADVANCE, dt);
}

void snowref_download(const SnowRef* s, float* pxm, int* pv, float* pFE, float* pFP) {
  if (!s->N) return;
  if (pxm) std::memcpy(pxm, s->pxm.data(), sizeof(vec4) * s->N);
  if (pv) std::memcpy(pv, s->pv.data(), sizeof(ivec4) * s->N);
  if (pFE) std::memcpy(pFE, s->pFE.data(), sizeof(mat4) * s->N);
  if (pFP) std::memcpy(pFP, s->pFP.data(), sizeof(mat4) * s->N);
}

// Per-particle G2P accumulators (pvn, pdvp0..2), N x ivec4 each.
void snowref_download_accumulators(const SnowRef* s, int* pvn, int* pd0, int* pd1, int* pd2) {
  if (!s->N) return;
  if (pvn) std::memcpy(pvn, s->pvn.data(), sizeof(ivec4) * s->N);
  if (pd0) std::memcpy(pd0, s->pd0.data(), sizeof(ivec4) * s->N);
  if (pd1) std::memcpy(pd1, s->pd1.data(), sizeof(ivec4) * s->N);
  if (pd2) std::memcpy(pd2, s->pd2.data(), sizeof(ivec4) * s->N);
}

// Grid buffers of the first G nodes: gv, gf (G x ivec4), gvn, gxm (G x vec4).
void snowref_download_grid(const SnowRef* s, int* gv, int* gf, float* gvn, float* gxm) {
  if (gv) std::memcpy(gv, s->gv.data(), sizeof(ivec4) * s->G);
  if (gf) std::memcpy(gf, s->gf.data(), sizeof(ivec4) * s->G);
  if (gvn) std::memcpy(gvn, s->gvn.data(), sizeof(vec4) * s->G);
  if (gxm) std::memcpy(gxm, s->gxm.data(), sizeof(vec4) * s->G);
}

// Colliders after rigidAdvance: cx (pos, type) n x vec4.
void snowref_download_colliders(const SnowRef* s, float* cx) {
  if (cx && s->ncoll) std::memcpy(cx, s->cx.data(), sizeof(vec4) * s->ncoll);
}

}  // extern "C"
