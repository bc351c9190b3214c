// CPU check of the stage runtime (no GPU): a source -> stage -> sink pipeline
// over a pool smaller than the stream, so back-pressure, in-order delivery,
// metadata propagation and the end-of-stream sentinel are all exercised.
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <thread>
#include <vector>

#include "glados_gb/Image.h"
#include "glados_gb/Pipeline.h"

struct MallocManager {
   using value_type = int;
   struct Deleter {
      void operator()(int* p) const { std::free(p); }
   };
   using pointer_type = std::unique_ptr<int, Deleter>;
   static pointer_type make_ptr(std::size_t n) { return pointer_type((int*)std::malloc(n * sizeof(int))); }
};
using Img = glados_gb::Image<MallocManager>;
using Pool = glados_gb::MemoryPool<MallocManager>;

struct Source {
   using output_type = Img;
   unsigned pool = Pool::instance()->registerStage(3, 16);
   int next = 0, total;
   explicit Source(int n) : total(n) {}
   Img loadImage() {
      if (next >= total) return Img();
      Img im = Pool::instance()->requestMemory(pool);  // blocks until a buffer comes back
      for (int i = 0; i < 16; ++i) im.data()[i] = next * 100 + i;
      im.setIdx(next);
      im.setPlane(next % 2);
      ++next;
      return im;
   }
};

struct Doubler {
   using input_type = Img;
   using output_type = Img;
   unsigned pool = Pool::instance()->registerStage(2, 16);
   glados_gb::Queue<Img> out;
   void process(Img&& in) {
      if (!in.valid()) {
         out.push(Img());
         return;
      }
      Img o = Pool::instance()->requestMemory(pool);
      for (int i = 0; i < 16; ++i) o.data()[i] = 2 * in.data()[i];
      o.setIdx(in.index());
      o.setPlane(in.plane());
      out.push(std::move(o));
   }
   Img wait() { return out.take(); }
};

struct Sink {
   using input_type = Img;
   int seen = 0, errors = 0;
   void saveImage(Img&& im) {
      if ((int)im.index() != seen || (int)im.plane() != seen % 2) ++errors;
      for (int i = 0; i < 16; ++i)
         if (im.data()[i] != 2 * (seen * 100 + i)) ++errors;
      ++seen;
   }
};

int main() {
   const int n = 200;
   glados_gb::Pipeline p;
   auto src = p.create<glados_gb::SourceStage<Source>>(n);
   auto mid = p.create<glados_gb::Stage<Doubler>>();
   auto snk = p.create<glados_gb::SinkStage<Sink>>();
   p.connect(src, mid);
   p.connect(mid, snk);
   p.run(src, mid, snk);
   p.wait();
   const bool pools_full = Pool::instance()->available(src->pool) == 3 && Pool::instance()->available(mid->pool) == 2;
   std::printf("seen=%d errors=%d pools_full=%d\n", snk->seen, snk->errors, (int)pools_full);
   return (snk->seen == n && snk->errors == 0 && pools_full) ? 0 : 1;
}
