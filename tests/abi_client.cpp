// abi_client.cpp — a C++ host that uses only include/gbrt.h and libgbrt.so,
// the way the renderer's GpuPerPixelRenderer would: parse a scene file,
// create the scene, render it with the renderer's options, render it again
// with the Metropolis renderer, and write the image. Built and run by
// tests/test_abi_client.py.
//
//   abi_client <scene file> <output image> <x samples> <y samples> <max depth>
// Prints one line "ok <paths> <mean of the film> <mean of the Metropolis film>".
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gbrt.h"

static int die(gbrt_ctx* ctx, const char* what) {
  std::fprintf(stderr, "%s: %s\n", what, gbrt_last_error(ctx));
  return 1;
}

int main(int argc, char** argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: abi_client scene image xs ys depth\n");
    return 2;
  }
  if (gbrt_abi_version() != GBRT_ABI_VERSION) return die(nullptr, "ABI version");
  gbrt_parsed_scene* ps = nullptr;
  char err[512];
  if (gbrt_parse_scene_file(argv[1], &ps, err, sizeof err) != GBRT_OK) {
    std::fprintf(stderr, "parse: %s\n", err);
    return 1;
  }
  gbrt_scene_desc desc;
  gbrt_camera cam;
  int32_t has_cam = 0;
  gbrt_parsed_scene_desc(ps, &desc, &cam, &has_cam);
  if (!has_cam) return die(nullptr, "scene without a camera");
  gbrt_ctx* ctx = nullptr;
  if (gbrt_ctx_create(0, &ctx) != GBRT_OK) return die(nullptr, "context");
  gbrt_scene* scene = nullptr;
  if (gbrt_scene_create(ctx, &desc, &scene) != GBRT_OK) return die(ctx, "scene");
  gbrt_parsed_scene_free(ps);  // the scene holds its own copy

  gbrt_render_params p = {};
  p.x_samples = std::atoi(argv[3]);
  p.y_samples = std::atoi(argv[4]);
  p.termination_prob = 0.5f;
  p.max_depth = std::atoi(argv[5]);
  p.seed = 1;
  p.semantics = GBRT_SEM_REFERENCE;
  std::vector<float> film(size_t(cam.width) * cam.height * 3);
  volatile int32_t stop = 0;
  gbrt_stats st;
  if (gbrt_render(scene, &cam, &p, film.data(), nullptr, nullptr, &stop, &st) != GBRT_OK) return die(ctx, "render");
  double mean = 0;
  for (float v : film) mean += v;
  mean /= double(film.size());

  gbrt_mlt_params mp = {};
  mp.mutations = 4;
  mp.bootstrap = 1000;
  mp.large_step_prob = 0.1f;
  mp.termination_prob = 0.5f;
  mp.chains = 1024;
  std::vector<float> mfilm(film.size());
  gbrt_chain_stats cs;
  if (gbrt_render_mlt(scene, &cam, &p, &mp, mfilm.data(), &cs) != GBRT_OK) return die(ctx, "render_mlt");
  double mmean = 0;
  for (float v : mfilm) mmean += v;
  mmean /= double(mfilm.size());

  if (gbrt_write_image(argv[2], film.data(), cam.width, cam.height, 2.2f) != GBRT_OK) return die(ctx, "write");
  gbrt_scene_destroy(scene);
  gbrt_ctx_destroy(ctx);
  std::printf("ok %llu %.6f %.6f\n", (unsigned long long)st.paths, mean, mmean);
  return 0;
}
