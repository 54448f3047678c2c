/* Minimal stand-in for the parts of boost.thread that the reference's
   MULTITHREADING.h names (thread, mutex::scoped_lock, this_thread::sleep). */
#pragma once
#include <chrono>
#include <mutex>
#include <thread>
namespace boost {
struct thread : std::thread { using std::thread::thread; };
struct mutex : std::mutex { typedef std::unique_lock<std::mutex> scoped_lock; };
namespace posix_time { inline std::chrono::microseconds microseconds(long n) { return std::chrono::microseconds(n); } }
namespace this_thread { template <class D> inline void sleep(D d) { std::this_thread::sleep_for(d); } }
}  // namespace boost
