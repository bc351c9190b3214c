// Thread-per-stage pipeline wiring with the reference's stage contract.
//
// A stage implementation provides input_type, output_type, a constructor,
// process(input_type&&) and wait() -> output_type (glados/pipeline/Stage.h:39-97).
// Stage<Impl> runs a push thread (input queue -> Impl::process) and a take
// thread (Impl::wait -> next stage); an invalid Image travels down the chain
// as the end-of-stream sentinel. SourceStage<Loader> calls loadImage() until
// it returns an invalid Image; SinkStage<Saver> hands every image to
// saveImage(). Pipeline::run starts every stage's thread, wait joins them.
#pragma once

#include <memory>
#include <thread>
#include <utility>
#include <vector>

#include "Queue.h"

namespace glados_gb {

template <class T>
class InputSide {
 public:
   void input(T&& t) { input_queue_.push(std::move(t)); }

 protected:
   Queue<T> input_queue_;
};

template <class T>
class OutputSide {
 public:
   void attach(InputSide<T>* next) { next_ = next; }

 protected:
   void output(T&& t) {
      if (next_) next_->input(std::move(t));
   }

 private:
   InputSide<T>* next_ = nullptr;
};

template <class Impl>
class Stage : public InputSide<typename Impl::input_type>,
              public OutputSide<typename Impl::output_type>,
              public Impl {
 public:
   using input_type = typename Impl::input_type;
   using output_type = typename Impl::output_type;

   template <typename... Args>
   explicit Stage(Args&&... args) : Impl(std::forward<Args>(args)...) {}

   void run() {
      std::thread push_thread{&Stage::push, this};
      std::thread take_thread{&Stage::take, this};
      push_thread.join();
      take_thread.join();
   }

 private:
   void push() {
      while (true) {
         auto img = this->input_queue_.take();
         const bool valid = img.valid();
         Impl::process(std::move(img));
         if (!valid) break;  // the sentinel has been forwarded to the implementation
      }
   }
   void take() {
      while (true) {
         auto result = Impl::wait();
         const bool valid = result.valid();
         this->output(std::move(result));
         if (!valid) break;
      }
   }
};

template <class Loader>
class SourceStage : public OutputSide<typename Loader::output_type>, public Loader {
 public:
   using output_type = typename Loader::output_type;
   template <typename... Args>
   explicit SourceStage(Args&&... args) : Loader(std::forward<Args>(args)...) {}
   void run() {
      while (true) {
         auto img = Loader::loadImage();
         const bool valid = img.valid();
         this->output(std::move(img));
         if (!valid) break;
      }
   }
};

template <class Saver>
class SinkStage : public InputSide<typename Saver::input_type>, public Saver {
 public:
   using input_type = typename Saver::input_type;
   template <typename... Args>
   explicit SinkStage(Args&&... args) : Saver(std::forward<Args>(args)...) {}
   void run() {
      while (true) {
         auto img = this->input_queue_.take();
         if (!img.valid()) break;
         Saver::saveImage(std::move(img));
      }
   }
};

class Pipeline {
 public:
   template <class S, typename... Args>
   std::shared_ptr<S> create(Args&&... args) {
      return std::make_shared<S>(std::forward<Args>(args)...);
   }
   template <class A, class B>
   void connect(const std::shared_ptr<A>& a, const std::shared_ptr<B>& b) {
      a->attach(b.get());
   }
   template <class... Stages>
   void run(const std::shared_ptr<Stages>&... stages) {
      (threads_.emplace_back([s = stages] { s->run(); }), ...);
   }
   void wait() {
      for (auto& t : threads_) t.join();
      threads_.clear();
   }

 private:
   std::vector<std::thread> threads_;
};

}  // namespace glados_gb
