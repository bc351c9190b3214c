// Bounded blocking queue between pipeline stages; push blocks while the queue
// holds `limit` items (0 = unbounded), take blocks while it is empty. Same
// contract as the reference's glados::Queue (glados/Queue.h:40-97).
#pragma once

#include <condition_variable>
#include <cstddef>
#include <mutex>
#include <queue>
#include <utility>

namespace glados_gb {

template <class Object>
class Queue {
 public:
   Queue() : limit_{10u} {}
   explicit Queue(std::size_t limit) : limit_{limit} {}

   template <class Item>
   void push(Item&& item) {
      std::unique_lock<std::mutex> lock{mutex_};
      if (limit_ != 0u) not_full_.wait(lock, [&] { return queue_.size() < limit_; });
      queue_.push(std::forward<Item>(item));
      not_empty_.notify_one();
   }

   Object take() {
      std::unique_lock<std::mutex> lock{mutex_};
      not_empty_.wait(lock, [&] { return !queue_.empty(); });
      Object ret = std::move(queue_.front());
      queue_.pop();
      not_full_.notify_one();
      return ret;
   }

   std::size_t size() const {
      std::lock_guard<std::mutex> lock{mutex_};
      return queue_.size();
   }

 private:
   const std::size_t limit_;
   mutable std::mutex mutex_;
   std::condition_variable not_empty_, not_full_;
   std::queue<Object> queue_;
};

}  // namespace glados_gb
