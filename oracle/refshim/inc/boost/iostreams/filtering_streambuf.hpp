// Header shim for the gzip step of the reference's writer (fomo-io.cpp:154-170).
// Boost.Iostreams is not installed here.  Building fomo-io.cpp needs the names
// to exist; running the gzip path in the shimmed build raises an error instead
// of writing a file.  The text and binary writers (fomo-io.cpp:26-150) do not
// use Boost and run unchanged.
#ifndef FOMO_REFSHIM_BOOST_IOSTREAMS_HPP
#define FOMO_REFSHIM_BOOST_IOSTREAMS_HPP
#include <ios>
#include <stdexcept>
namespace boost {
namespace iostreams {
struct input {};
struct gzip_compressor {};
template <typename Mode>
class filtering_streambuf {
 public:
  template <typename T>
  void push(T const&) {}
  template <typename T>
  void push(T&) {}
};
template <typename Source, typename Sink>
std::streamsize copy(Source&, Sink&) {
  throw std::runtime_error("gzip output is not available in the shimmed reference build");
}
}  // namespace iostreams
}  // namespace boost
#endif
