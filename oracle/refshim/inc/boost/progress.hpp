// Header shim: boost::progress_display only draws a progress bar on stdout in
// the reference (fomo-nearestneighbour.cpp:141,228; fomo-thomson.cpp:262,341).
// It has no effect on any computed value, so the shim counts silently.
#ifndef FOMO_REFSHIM_BOOST_PROGRESS_HPP
#define FOMO_REFSHIM_BOOST_PROGRESS_HPP
#include <iostream>  // the real header includes <iostream>
namespace boost {
class progress_display {
 public:
  explicit progress_display(unsigned long expected) : count_(0), expected_(expected) {}
  unsigned long operator++() { return ++count_; }
  unsigned long count() const { return count_; }
  unsigned long expected_count() const { return expected_; }

 private:
  unsigned long count_;
  unsigned long expected_;
};
}  // namespace boost
#endif
