// Minimal stand-in for the glog logging API, written for this project so that
// the reference's sources compile without the real library. Test
// infrastructure only: it is used by the oracle build, never by the product.
//
// Provided: LOG(severity), VLOG(n), CHECK / CHECK_xx, DCHECK / DCHECK_xx and
// google::InitGoogleLogging / google::InstallFailureSignalHandler. A failed
// CHECK or LOG(FATAL) prints its message and aborts, like glog.
#pragma once

#include <cstdlib>
#include <cstring> // the real glog header brings in <cstring> too
#include <iostream>
#include <limits>
#include <sstream>

namespace google {
inline void InitGoogleLogging(const char *) {}
inline void InstallFailureSignalHandler() {}
} // namespace google

namespace shim_glog {

enum Severity { INFO = 0, WARNING = 1, ERROR = 2, FATAL = 3 };

// Verbosity threshold for LOG(INFO)/VLOG output; messages are dropped unless
// the environment variable SHIM_GLOG_VERBOSE is set.
inline bool Verbose() {
  static const bool v = std::getenv("SHIM_GLOG_VERBOSE") != nullptr;
  return v;
}

class Message {
public:
  Message(const char *file, int line, int severity)
      : severity_(severity), enabled_(severity >= ERROR || Verbose()) {
    if (enabled_) {
      os_ << file << ":" << line << "] ";
    }
  }
  ~Message() {
    if (enabled_) {
      std::cerr << os_.str() << std::endl;
    }
    if (severity_ == FATAL) {
      std::abort();
    }
  }
  std::ostream &stream() { return os_; }

private:
  int severity_;
  bool enabled_;
  std::ostringstream os_;
};

// Swallows the stream of a CHECK that passed.
struct Voidify {
  void operator&(std::ostream &) {}
};

} // namespace shim_glog

#define LOG(sev) shim_glog::Message(__FILE__, __LINE__, shim_glog::sev).stream()
#define VLOG(n) shim_glog::Message(__FILE__, __LINE__, shim_glog::INFO).stream()

#define CHECK(cond)                                                            \
  (cond) ? (void)0                                                             \
         : shim_glog::Voidify() &                                              \
               shim_glog::Message(__FILE__, __LINE__, shim_glog::FATAL)        \
                       .stream()                                               \
                   << "Check failed: " #cond " "

#define SHIM_CHECK_OP(a, b, op)                                                \
  ((a)op(b)) ? (void)0                                                         \
             : shim_glog::Voidify() &                                          \
                   shim_glog::Message(__FILE__, __LINE__, shim_glog::FATAL)    \
                           .stream()                                           \
                       << "Check failed: " #a " " #op " " #b " (" << (a)       \
                       << " vs " << (b) << ") "

#define CHECK_EQ(a, b) SHIM_CHECK_OP(a, b, ==)
#define CHECK_NE(a, b) SHIM_CHECK_OP(a, b, !=)
#define CHECK_LT(a, b) SHIM_CHECK_OP(a, b, <)
#define CHECK_LE(a, b) SHIM_CHECK_OP(a, b, <=)
#define CHECK_GT(a, b) SHIM_CHECK_OP(a, b, >)
#define CHECK_GE(a, b) SHIM_CHECK_OP(a, b, >=)

#ifdef NDEBUG
#define SHIM_DCHECK_NOP(...)                                                   \
  while (false)                                                                \
  shim_glog::Message(__FILE__, __LINE__, shim_glog::INFO).stream()
#define DCHECK(cond) SHIM_DCHECK_NOP()
#define DCHECK_EQ(a, b) SHIM_DCHECK_NOP()
#define DCHECK_NE(a, b) SHIM_DCHECK_NOP()
#define DCHECK_LT(a, b) SHIM_DCHECK_NOP()
#define DCHECK_LE(a, b) SHIM_DCHECK_NOP()
#define DCHECK_GT(a, b) SHIM_DCHECK_NOP()
#define DCHECK_GE(a, b) SHIM_DCHECK_NOP()
#else
#define DCHECK(cond) CHECK(cond)
#define DCHECK_EQ(a, b) CHECK_EQ(a, b)
#define DCHECK_NE(a, b) CHECK_NE(a, b)
#define DCHECK_LT(a, b) CHECK_LT(a, b)
#define DCHECK_LE(a, b) CHECK_LE(a, b)
#define DCHECK_GT(a, b) CHECK_GT(a, b)
#define DCHECK_GE(a, b) CHECK_GE(a, b)
#endif
