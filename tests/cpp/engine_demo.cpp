// Uses the C++ host layer (include/narval_engine.hpp) the way reference code would:
// SceneReader -> GpuScene -> OfflineEngine::coreLoop. Without --render it only loads the
// scene (no GPU needed) and prints its settings.
#include <cstdio>
#include <cstring>

#include "narval_engine.hpp"

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: engine_demo scene.json [--render out.ppm]\n");
    return 2;
  }
  try {
    narvalgb::SceneReader reader(argv[1]);
    const ne_settings& s = reader.getSettings();
    std::printf("settings %d %d %d %d\n", s.width, s.height, s.spp, s.bounces);
    if (argc >= 4 && std::strcmp(argv[2], "--render") == 0) {
      narvalgb::GpuScene scene(reader);
      narvalgb::OfflineEngine engine(scene, 1, false);
      ne_render_stats st = engine.coreLoop(argv[3]);
      std::printf("rendered %llu paths in %.3f ms\n", (unsigned long long)st.paths, st.kernel_ms);
      narvalgb::VolumetricPathIntegrator integrator(scene, 1);
      ne_ray r = {{0, 1, -2}, {0, 0, 1}};
      narvalgb::Vec3 L = integrator.Li(r, ne_path_key{0, 0});
      std::printf("Li %g %g %g\n", L.x, L.y, L.z);
    }
  } catch (const narvalgb::Error& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
