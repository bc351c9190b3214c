// Source and sink stages for the pipeline example: the reference's
// per-module raw data files in, float TIFF stacks out.
//
//   OfflineLoader  RISA/risaLib/src/Loader/OfflineLoader.cu:56-95: module file
//                  <dataInputPath>/<dataFileName><i><dataFileEnding> (i from 1)
//                  holds consecutive blocks of n_proj x (n_det / n_modules)
//                  uint16 values; block b is frame b / n_planes of plane
//                  b % n_planes. Frames are emitted module-major, as read.
//   TiffSaver      RISA/risaLib/src/Saver/OfflineSaver.cu:102-178: one
//                  multi-page 32-bit float TIFF per plane,
//                  <outputPath>/<outputFileName>_plane<k>.tif, pages in the
//                  order the images arrive, with the latency bookkeeping of
//                  the reference (min/max milliseconds since loading).
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../glados_gb/Image.h"
#include "Packets.h"
#include "Stages.h"

namespace risa_gb {

// Packet layout of the detector modules from the configuration keys the
// reference's receiver reads (ReceiverModule.cpp:139-163).
inline PacketLayout packet_layout(const Config& cfg) {
   PacketLayout L;
   L.modules = cfg.geometry.n_modules;
   L.det_per_module = (int)cfg.integer("numberOfDetectorsPerModule",
                                       L.modules > 0 ? cfg.geometry.n_fan_det / L.modules : 0);
   L.proj = cfg.geometry.n_fan_proj;
   L.proj_per_packet = (int)cfg.integer("numberOfProjectionsPerPacket", L.proj);
   L.ring = (int)cfg.integer("inputBufferSize", 32);
   return L;
}

// Source stage of the online mode: the reference's Receiver::loadImage
// (Receiver.cpp:66-86) over a FrameAssembler fed by any transport. Each
// complete frame is copied from the ring into a pooled module-major image
// (the OfflineLoader's output layout) and released; the stream ends (invalid
// image) when the assembler finishes or no frame completes within `timeout`
// seconds (config key timeout, as the reference's receiver modules).
class OnlineLoader {
 public:
   using manager_type = cuda::RawHostManager;
   using output_type = glados_gb::Image<manager_type>;

   OnlineLoader(const std::string& config_file, FrameAssembler& frames) : cfg_(config_file), fa_(frames) {
      const PacketLayout& L = fa_.layout();
      if (L.frame_values() != (size_t)cfg_.geometry.n_fan_proj * cfg_.geometry.n_fan_det)
         throw std::runtime_error("OnlineLoader: packet layout does not match the geometry");
      timeout_ = (double)cfg_.integer("timeout", 10);
      pool_ = glados_gb::MemoryPool<manager_type>::instance()->registerStage(8, L.frame_values());
   }
   ~OnlineLoader() { glados_gb::MemoryPool<manager_type>::instance()->freeMemory(pool_); }

   output_type loadImage() {
      uint64_t index = 0;
      const uint16_t* frame = nullptr;
      if (!fa_.next(&index, &frame, timeout_)) return output_type();
      output_type img = glados_gb::MemoryPool<manager_type>::instance()->requestMemory(pool_);
      std::copy(frame, frame + fa_.layout().frame_values(), img.data());
      fa_.release(index);
      img.setIdx((size_t)index);
      img.setPlane((size_t)(index % (uint64_t)cfg_.geometry.n_planes));
      img.setStart(std::chrono::high_resolution_clock::now());
      return img;
   }

 private:
   Config cfg_;
   FrameAssembler& fa_;
   double timeout_ = 10.0;
   int pool_ = 0;
};

class OfflineLoader {
 public:
   using manager_type = cuda::RawHostManager;
   using output_type = glados_gb::Image<manager_type>;

   explicit OfflineLoader(const std::string& config_file) : cfg_(config_file) {
      const auto& g = cfg_.geometry;
      modules_ = g.n_modules;
      if (modules_ < 1 || g.n_fan_det % modules_) throw std::runtime_error("OfflineLoader: bad module count");
      frames_ = (long)cfg_.integer("numberOfDataFrames", 0) * g.n_planes;
      const std::string prefix = cuda::with_slash(cfg_.str("dataInputPath")) + cfg_.str("dataFileName");
      const std::string ending = cfg_.str("dataFileEnding", ".fx");
      for (int m = 1; m <= modules_; ++m) {
         const std::string path = prefix + std::to_string(m) + ending;
         FILE* f = std::fopen(path.c_str(), "rb");
         if (!f) throw std::runtime_error("OfflineLoader: cannot open " + path);
         files_.push_back(f);
      }
      elems_ = (size_t)g.n_fan_proj * g.n_fan_det;
      pool_ = glados_gb::MemoryPool<manager_type>::instance()->registerStage(
          (int)cfg_.integer("inputBufferSize", 32) > 64 ? 64 : (int)cfg_.integer("inputBufferSize", 32), elems_);
   }
   ~OfflineLoader() {
      for (FILE* f : files_) std::fclose(f);
      glados_gb::MemoryPool<manager_type>::instance()->freeMemory(pool_);
   }

   output_type loadImage() {
      if (index_ >= frames_) return output_type();
      const auto& g = cfg_.geometry;
      const size_t block = (size_t)g.n_fan_proj * (g.n_fan_det / modules_);
      output_type img = glados_gb::MemoryPool<manager_type>::instance()->requestMemory(pool_);
      for (int m = 0; m < modules_; ++m) {
         std::fseek(files_[m], (long)(index_ * block * sizeof(uint16_t)), SEEK_SET);
         if (std::fread(img.data() + (size_t)m * block, sizeof(uint16_t), block, files_[m]) != block)
            throw std::runtime_error("OfflineLoader: short read");
      }
      img.setIdx((size_t)index_);
      img.setPlane((size_t)(index_ % g.n_planes));
      img.setStart(std::chrono::high_resolution_clock::now());
      ++index_;
      return img;
   }

 private:
   Config cfg_;
   int modules_ = 1;
   long frames_ = 0, index_ = 0;
   size_t elems_ = 0;
   unsigned pool_ = 0;
   std::vector<FILE*> files_;
};

// Minimal multi-page little-endian TIFF writer for 32-bit float images.
class FloatTiffWriter {
 public:
   FloatTiffWriter(const std::string& path, int width, int height) : w_(width), h_(height) {
      f_ = std::fopen(path.c_str(), "wb");
      if (!f_) throw std::runtime_error("TIFF: cannot create " + path);
      const uint8_t hdr[8] = {'I', 'I', 42, 0, 8, 0, 0, 0};  // first IFD offset patched later
      std::fwrite(hdr, 1, 8, f_);
      next_ptr_pos_ = 4;
   }
   ~FloatTiffWriter() {
      if (f_) std::fclose(f_);
   }
   void append(const float* data) {
      const uint32_t bytes = (uint32_t)((size_t)w_ * h_ * 4);
      const uint32_t data_pos = (uint32_t)std::ftell(f_);
      std::fwrite(data, 4, (size_t)w_ * h_, f_);
      const uint32_t ifd_pos = (uint32_t)std::ftell(f_);
      // entries: tag, type (3 SHORT, 4 LONG), count, value
      const uint16_t n = 10;
      struct E { uint16_t tag, type; uint32_t count, value; };
      const E es[n] = {{256, 4, 1, (uint32_t)w_}, {257, 4, 1, (uint32_t)h_}, {258, 3, 1, 32},
                       {259, 3, 1, 1},           {262, 3, 1, 1},           {273, 4, 1, data_pos},
                       {277, 3, 1, 1},           {278, 4, 1, (uint32_t)h_}, {279, 4, 1, bytes},
                       {339, 3, 1, 3}};
      std::fwrite(&n, 2, 1, f_);
      for (const E& e : es) {
         std::fwrite(&e.tag, 2, 1, f_);
         std::fwrite(&e.type, 2, 1, f_);
         std::fwrite(&e.count, 4, 1, f_);
         std::fwrite(&e.value, 4, 1, f_);
      }
      const uint32_t zero = 0;
      const long ptr_pos = std::ftell(f_);
      std::fwrite(&zero, 4, 1, f_);
      // link the previous IFD (or the header) to this one
      std::fseek(f_, next_ptr_pos_, SEEK_SET);
      std::fwrite(&ifd_pos, 4, 1, f_);
      std::fseek(f_, 0, SEEK_END);
      next_ptr_pos_ = ptr_pos;
      ++pages_;
   }
   int pages() const { return pages_; }

 private:
   FILE* f_ = nullptr;
   int w_, h_;
   long next_ptr_pos_ = 4;
   int pages_ = 0;
};

class TiffSaver {
 public:
   using manager_type = cuda::FloatHostManager;
   using input_type = glados_gb::Image<manager_type>;

   explicit TiffSaver(const std::string& config_file) : cfg_(config_file) {
      const auto& g = cfg_.geometry;
      const std::string dir = cuda::with_slash(cfg_.str("outputPath", "./"));
      const std::string name = cfg_.str("outputFileName", "reco");
      for (int k = 0; k < g.n_planes; ++k)
         writers_.emplace_back(new FloatTiffWriter(dir + name + "_plane" + std::to_string(k) + ".tif",
                                                   g.n_pixels, g.n_pixels));
   }
   void saveImage(input_type&& img) {
      const double ms = img.duration();
      min_latency_ = std::min(min_latency_, ms);
      max_latency_ = std::max(max_latency_, ms);
      writers_.at(img.plane())->append(img.data());
      ++saved_;
   }
   long saved() const { return saved_; }
   double min_latency_ms() const { return min_latency_; }
   double max_latency_ms() const { return max_latency_; }

 private:
   Config cfg_;
   std::vector<std::unique_ptr<FloatTiffWriter>> writers_;
   long saved_ = 0;
   double min_latency_ = std::numeric_limits<double>::max(), max_latency_ = 0.0;
};

}  // namespace risa_gb
