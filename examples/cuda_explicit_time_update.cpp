// The drop-in at the reference's MPMPhysicEngine seam, standalone: a class
// with the shape of the reference's TimeUpdate subclasses
// (src/snow/simulation/timeUpdate/timeUpdate.hpp:10-18: construct from the
// scene, init(), update(double dt)) that forwards to the C ABI of
// include/snow_mpm.h. A reference build would derive it from TimeUpdate and
// fill snow_params / snow_collider from its PhysicalScene; here a snowball
// in the reference's default world (defines.hpp) stands in for the scene.
//
// CudaSemiImplicitTimeUpdate does the same for the reference's
// SemiImplicitTimeUpdate (semiimplicittimeupdate.hpp:6-12, empty there): the
// scene's parameters ask for the semi-implicit velocity update.
//
//   g++ -std=c++17 -I include examples/cuda_explicit_time_update.cpp \
//       -L snow_gb300/_build -lsnow_gb300 -Wl,-rpath,snow_gb300/_build -o explicit_step
//   ./explicit_step [steps] [--semi-implicit]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "snow_mpm.h"

namespace {

struct PhysicalScene {  // what the reference's PhysicalScene carries for the step
  snow_params params;
  std::vector<snow_collider> colliders;
  std::vector<float> x, v, m;  // N x 3, N x 3, N
};

class CudaExplicitTimeUpdate {
 public:
  explicit CudaExplicitTimeUpdate(PhysicalScene&& s) : scene_(std::move(s)) {}
  virtual ~CudaExplicitTimeUpdate() {
    snow_scene_destroy(sim_);
    snow_ctx_destroy(ctx_);
  }

  // ExplicitTimeUpdate::init (explicittimeupdate.cpp:4-34): buffers, grid
  // mass, particle volumes.
  bool init() {
    if (snow_ctx_create(0, 0, &ctx_) != SNOW_OK) return fail("snow_ctx_create");
    if (snow_scene_create(ctx_, &scene_.params, scene_.colliders.data(), (int)scene_.colliders.size(), 0, &sim_))
      return fail("snow_scene_create");
    const size_t n = scene_.m.size();
    if (snow_scene_upload(sim_, scene_.x.data(), scene_.v.data(), scene_.m.data(), nullptr, nullptr, n))
      return fail("snow_scene_upload");
    if (snow_scene_init(sim_)) return fail("snow_scene_init");
    return true;
  }

  // ExplicitTimeUpdate::update (explicittimeupdate.cpp:36-63): one step.
  bool update(double dt) { return snow_scene_step(sim_, dt, 1) == SNOW_OK || fail("snow_scene_step"); }

  bool stats(snow_stats* out) { return snow_scene_stats(sim_, out) == SNOW_OK || fail("snow_scene_stats"); }

 protected:
  bool fail(const char* what) {
    std::fprintf(stderr, "%s failed: %s\n", what, ctx_ ? snow_last_error(ctx_) : "no context");
    return false;
  }
  PhysicalScene scene_;
  snow_ctx* ctx_ = nullptr;
  snow_scene* sim_ = nullptr;
};

// SemiImplicitTimeUpdate: each update solves (M + beta dt^2 K) v = M v* on
// the grid (conjugate residuals) before G2P.
class CudaSemiImplicitTimeUpdate : public CudaExplicitTimeUpdate {
 public:
  explicit CudaSemiImplicitTimeUpdate(PhysicalScene&& s, float beta = 1.0f)
      : CudaExplicitTimeUpdate(with_beta(std::move(s), beta)) {}
  bool report(snow_solver_report* out) {
    return snow_scene_solver_report(sim_, out) == SNOW_OK || fail("snow_scene_solver_report");
  }

 private:
  static PhysicalScene with_beta(PhysicalScene&& s, float beta) {
    s.params.implicit_beta = beta;
    s.params.implicit_tolerance = 1e-5f;
    s.params.implicit_max_iters = 50;
    return std::move(s);
  }
};

// A snowball of radius 0.3 m above the ground of the default world, seeded
// jittered lattice at 8 particles per cell, dropped at 2 m/s.
PhysicalScene snowball() {
  PhysicalScene s;
  snow_params_default(&s.params);  // defines.hpp world: grid, spacing, walls
  s.params.mode = SNOW_MODE_FAST;
  // the snowball material of the reference's snowball-drop scene
  s.params.young = 1.4e5f;
  s.params.poisson = 0.2f;
  s.params.hardening = 10.0f;
  s.params.crit_compression = 2.5e-2f;
  s.params.crit_stretch = 7.5e-3f;
  snow_collider walls[6];
  const int nw = snow_default_walls(&s.params, walls);
  s.colliders.assign(walls, walls + nw);
  const float h = s.params.grid_spacing;
  const float c[3] = {s.params.grid_pos[0] + 100 * h, s.params.grid_pos[1] + 40 * h, s.params.grid_pos[2] + 100 * h};
  std::mt19937 rng(5);
  std::uniform_real_distribution<float> jitter(-0.125f * h, 0.125f * h);
  const float r = 0.3f;
  for (float z = c[2] - r; z <= c[2] + r; z += 0.5f * h)
    for (float y = c[1] - r; y <= c[1] + r; y += 0.5f * h)
      for (float x = c[0] - r; x <= c[0] + r; x += 0.5f * h) {
        const float d2 = (x - c[0]) * (x - c[0]) + (y - c[1]) * (y - c[1]) + (z - c[2]) * (z - c[2]);
        if (d2 > r * r) continue;
        s.x.insert(s.x.end(), {x + jitter(rng), y + jitter(rng), z + jitter(rng)});
        s.v.insert(s.v.end(), {0.0f, -2.0f, 0.0f});
        s.m.push_back(400.0f * h * h * h / 8.0f);
      }
  return s;
}

}  // namespace

int main(int argc, char** argv) {
  const int steps = argc > 1 ? std::atoi(argv[1]) : 100;
  const bool semi = argc > 2 && std::string(argv[2]) == "--semi-implicit";
  PhysicalScene scene = snowball();
  const size_t n = scene.m.size();
  // MPMPhysicEngine's member
  CudaSemiImplicitTimeUpdate* si = semi ? new CudaSemiImplicitTimeUpdate(std::move(scene)) : nullptr;
  CudaExplicitTimeUpdate* integration = si ? si : new CudaExplicitTimeUpdate(std::move(scene));
  int rc = 0;
  snow_stats before{}, after{};
  if (!integration->init() || !integration->stats(&before)) rc = 1;
  for (int i = 0; i < steps && rc == 0; i++)
    if (!integration->update(1e-3)) rc = 1;
  if (rc == 0 && !integration->stats(&after)) rc = 1;
  if (rc == 0) {
    std::printf("%s particles %zu steps %d centre of mass y %.6f -> %.6f nonfinite %llu\n",
                semi ? "semi-implicit" : "explicit", n, steps, before.center_of_mass[1], after.center_of_mass[1],
                (unsigned long long)after.nonfinite);
    snow_solver_report rep{};
    if (si && si->report(&rep))
      std::printf("last solve: %d iterations, residual %.3g\n", rep.iterations, rep.residual);
    rc = after.nonfinite == 0 && after.center_of_mass[1] < before.center_of_mass[1] ? 0 : 2;
  }
  delete integration;
  return rc;
}
