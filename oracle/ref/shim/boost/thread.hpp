// Build-only stand-in for the few boost::thread facilities the reference estimator uses
// (thread from a bound callable, join, mutex, mutex::scoped_lock, bind), mapped onto the
// C++11 standard library. Used only to compile the reference CPU path as a test oracle.
#ifndef ORACLE_SHIM_BOOST_THREAD_HPP
#define ORACLE_SHIM_BOOST_THREAD_HPP
#include <thread>
#include <mutex>
#include <functional>
namespace boost {
class mutex : public std::mutex {
 public:
  typedef std::lock_guard<std::mutex> scoped_lock;
};
class thread {
 public:
  template <class F> explicit thread(F f) : t_(f) {}
  void join() { t_.join(); }
 private:
  std::thread t_;
};
using std::bind;
}  // namespace boost
#endif
