// C ABI of the online input side: risa_gb_assembler_* over FrameAssembler
// (risa_gb300/cpp/risa_gb/Packets.h). Host code only; no CUDA calls.
#include <memory>
#include <new>
#include <stdexcept>

#include "../cpp/risa_gb/Packets.h"
#include "risa_gb_internal.h"

using namespace risa_gb;

struct risa_gb_assembler {
   std::unique_ptr<FrameAssembler> fa;
};

extern "C" risa_gb_status risa_gb_assembler_create(const risa_gb_packet_layout* l, uint16_t* ring, int skip_lag,
                                                   int completion, risa_gb_assembler** out) {
   if (!out) return fail(RISA_GB_EINVAL, "assembler_create: out is NULL");
   *out = nullptr;
   if (!l || l->struct_size != sizeof(risa_gb_packet_layout))
      return fail(RISA_GB_EINVAL, "assembler_create: layout is NULL or its struct_size does not match");
   if (!ring) return fail(RISA_GB_EINVAL, "assembler_create: ring is NULL");
   if (completion != RISA_GB_COMPLETION_EXACT && completion != RISA_GB_COMPLETION_LAST_PART)
      return fail(RISA_GB_EINVAL, "assembler_create: unknown completion rule");
   if (skip_lag < 0) return fail(RISA_GB_EINVAL, "assembler_create: negative skip_lag");
   PacketLayout L;
   L.modules = l->modules;
   L.det_per_module = l->det_per_module;
   L.proj = l->proj;
   L.proj_per_packet = l->proj_per_packet;
   L.ring = l->ring;
   std::unique_ptr<risa_gb_assembler> h(new (std::nothrow) risa_gb_assembler());
   if (!h) return fail(RISA_GB_ENOMEM, "assembler_create: host allocation failed");
   try {
      h->fa.reset(new FrameAssembler(L, ring, skip_lag,
                                     completion == RISA_GB_COMPLETION_LAST_PART ? Completion::last_part
                                                                                : Completion::exact));
   } catch (const std::invalid_argument& e) {
      return fail(RISA_GB_EINVAL, std::string("assembler_create: ") + e.what());
   } catch (const std::bad_alloc&) {
      return fail(RISA_GB_ENOMEM, "assembler_create: host allocation failed");
   }
   *out = h.release();
   return RISA_GB_OK;
}

extern "C" int risa_gb_assembler_ingest(risa_gb_assembler* h, int module, const void* packet, size_t bytes) {
   if (!h) return fail(RISA_GB_EINVAL, "assembler_ingest: null handle");
   switch (h->fa->ingest(module, static_cast<const uint8_t*>(packet), bytes)) {
      case Ingest::accepted: return RISA_GB_INGEST_ACCEPTED;
      case Ingest::duplicate: return RISA_GB_INGEST_DUPLICATE;
      case Ingest::malformed: return RISA_GB_INGEST_MALFORMED;
      case Ingest::stale: return RISA_GB_INGEST_STALE;
      case Ingest::ring_full: return RISA_GB_INGEST_RING_FULL;
   }
   return RISA_GB_INGEST_MALFORMED;
}

extern "C" int risa_gb_assembler_next(risa_gb_assembler* h, double timeout_s, uint64_t* index, int* slot) {
   if (!h || !index || !slot) return fail(RISA_GB_EINVAL, "assembler_next: null argument");
   const uint16_t* frame = nullptr;
   if (!h->fa->next(index, &frame, timeout_s)) return 0;
   *slot = (int)(*index % (uint64_t)h->fa->layout().ring);
   return 1;
}

extern "C" risa_gb_status risa_gb_assembler_release(risa_gb_assembler* h, uint64_t index) {
   if (!h) return fail(RISA_GB_EINVAL, "assembler_release: null handle");
   h->fa->release(index);
   return RISA_GB_OK;
}

extern "C" risa_gb_status risa_gb_assembler_finish(risa_gb_assembler* h) {
   if (!h) return fail(RISA_GB_EINVAL, "assembler_finish: null handle");
   h->fa->finish();
   return RISA_GB_OK;
}

extern "C" risa_gb_status risa_gb_assembler_stats(risa_gb_assembler* h, uint64_t* skipped, uint64_t* abandoned,
                                                  uint64_t* duplicates) {
   if (!h) return fail(RISA_GB_EINVAL, "assembler_stats: null handle");
   if (skipped) *skipped = h->fa->skipped();
   if (abandoned) *abandoned = h->fa->abandoned();
   if (duplicates) *duplicates = h->fa->duplicates();
   return RISA_GB_OK;
}

extern "C" risa_gb_status risa_gb_assembler_destroy(risa_gb_assembler* h) {
   delete h;
   return RISA_GB_OK;
}
