// Streaming reconstruction pipeline driven by one configuration file, the
// counterpart of the reference's example application (RISA/example/main.cpp:70-162):
//
//   OfflineLoader -> H2D -> Reordering -> [DetectorInterpolation] -> Attenuation
//     -> Fan2Para -> Filter -> Backprojection -> [Masking] -> D2H -> TiffSaver
//
// DetectorInterpolation runs when the config sets gb_defects = true, Masking
// when gb_masking = true. With --batched the same frames go through the
// whole-chain engine instead (risa_gb_fbp_run_host: batched launches replayed
// from CUDA graphs, copies overlapped with compute).
//
//   risa_gb_pipeline <config file> [--batched]
#include <chrono>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "../glados_gb/Pipeline.h"
#include "../risa_gb/IO.h"
#include "../risa_gb/Stages.h"

namespace {

int run_stages(const std::string& config) {
   using namespace risa_gb;
   using namespace risa_gb::cuda;
   Config cfg(config);
   const bool defects = cfg.params.defects != 0;
   const bool masking = cfg.params.masking != 0;
   glados_gb::Pipeline pipeline;
   auto source = pipeline.create<glados_gb::SourceStage<OfflineLoader>>(config);
   auto h2d = pipeline.create<glados_gb::Stage<H2D>>(config);
   auto reordering = pipeline.create<glados_gb::Stage<Reordering>>(config);
   auto interp = defects ? pipeline.create<glados_gb::Stage<DetectorInterpolation>>(config) : nullptr;
   auto attenuation = pipeline.create<glados_gb::Stage<Attenuation>>(config);
   auto fan2para = pipeline.create<glados_gb::Stage<Fan2Para>>(config);
   auto filter = pipeline.create<glados_gb::Stage<Filter>>(config);
   auto bp = pipeline.create<glados_gb::Stage<Backprojection>>(config);
   auto mask = masking ? pipeline.create<glados_gb::Stage<Masking>>(config) : nullptr;
   auto d2h = pipeline.create<glados_gb::Stage<D2H>>(config);
   auto sink = pipeline.create<glados_gb::SinkStage<TiffSaver>>(config);

   pipeline.connect(source, h2d);
   pipeline.connect(h2d, reordering);
   if (interp) {
      pipeline.connect(reordering, interp);
      pipeline.connect(interp, attenuation);
   } else {
      pipeline.connect(reordering, attenuation);
   }
   pipeline.connect(attenuation, fan2para);
   pipeline.connect(fan2para, filter);
   pipeline.connect(filter, bp);
   if (mask) {
      pipeline.connect(bp, mask);
      pipeline.connect(mask, d2h);
   } else {
      pipeline.connect(bp, d2h);
   }
   pipeline.connect(d2h, sink);

   const auto t0 = std::chrono::steady_clock::now();
   pipeline.run(source, h2d, reordering, attenuation, fan2para, filter, bp, d2h, sink);
   if (interp) pipeline.run(interp);
   if (mask) pipeline.run(mask);
   pipeline.wait();
   const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
   std::printf("{\"mode\": \"stages\", \"images\": %ld, \"seconds\": %.6f, \"images_per_s\": %.3f, "
               "\"lost\": %ld, \"latency_ms\": [%.3f, %.3f]}\n",
               sink->saved(), s, sink->saved() / s, h2d->lost(), sink->min_latency_ms(), sink->max_latency_ms());
   return 0;
}

int run_batched(const std::string& config) {
   using namespace risa_gb;
   Config cfg(config);
   const auto& g = cfg.geometry;
   const int n_ref = (int)cfg.integer("numberOfReferenceFrames", 1);
   const int n_dark = (int)cfg.integer("numberOfDarkFrames", 1);
   auto ref = cuda::read_module_files(cuda::with_slash(cfg.str("referenceInputPath")) +
                                          "ref_empty_tomograph_repaired_DetModNr_",
                                      ".fx", g.n_modules, n_ref, g.n_planes, g.n_fan_proj, g.n_fan_det);
   std::vector<uint16_t> dark;
   const std::string dark_dir = cfg.str("darkInputPath");
   if (!dark_dir.empty())
      dark = cuda::read_module_files(cuda::with_slash(dark_dir) + "dark_192.168.100_DetModNr_", ".fx",
                                     g.n_modules, n_dark, g.n_planes, g.n_fan_proj, g.n_fan_det);
   const int frames = (int)cfg.integer("numberOfDataFrames", 0);
   const int n = frames * g.n_planes;
   // data frames, module-major as stored; the engine fuses the reordering
   risa_gb_params p = cfg.params;
   p.module_major = 1;
   std::vector<uint16_t> raw;
   {
      OfflineLoader loader(config);
      raw.resize((size_t)n * g.n_fan_proj * g.n_fan_det);
      for (int i = 0; i < n; ++i) {
         auto img = loader.loadImage();
         std::memcpy(raw.data() + (size_t)i * g.n_fan_proj * g.n_fan_det, img.data(),
                     sizeof(uint16_t) * g.n_fan_proj * g.n_fan_det);
      }
   }
   const int batch = (int)cfg.integer("gb_batch", 32) / g.n_planes * g.n_planes;
   risa_gb_fbp* h = nullptr;
   check(risa_gb_fbp_create(&g, &p, ref.data(), n_ref, dark.empty() ? nullptr : dark.data(),
                            dark.empty() ? 0 : n_dark, batch > 0 ? batch : g.n_planes, &h),
         "fbp_create");
   std::vector<float> img((size_t)n * g.n_pixels * g.n_pixels);
   const auto t0 = std::chrono::steady_clock::now();
   check(risa_gb_fbp_run_host(h, raw.data(), img.data(), n, RISA_GB_PLANES_INTERLEAVED), "fbp_run_host");
   const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
   risa_gb_fbp_destroy(h);
   const std::string dir = cuda::with_slash(cfg.str("outputPath", "./"));
   const std::string name = cfg.str("outputFileName", "reco");
   for (int k = 0; k < g.n_planes; ++k) {
      FloatTiffWriter w(dir + name + "_plane" + std::to_string(k) + ".tif", g.n_pixels, g.n_pixels);
      for (int i = k; i < n; i += g.n_planes) w.append(img.data() + (size_t)i * g.n_pixels * g.n_pixels);
   }
   std::printf("{\"mode\": \"batched\", \"images\": %d, \"seconds\": %.6f, \"images_per_s\": %.3f}\n", n, s,
               n / s);
   return 0;
}

}  // namespace

int main(int argc, char** argv) {
   if (argc < 2) {
      std::cerr << "usage: risa_gb_pipeline <config file> [--batched]" << std::endl;
      return 1;
   }
   const std::string config = argv[1];
   const bool batched = argc > 2 && std::strcmp(argv[2], "--batched") == 0;
   try {
      return batched ? run_batched(config) : run_stages(config);
   } catch (const std::exception& e) {
      std::cerr << "A runtime error occurred: " << e.what() << std::endl;
      return 2;
   }
}
