// Header shim for the subset of Boost.Geometry that the reference's
// nearest-neighbour and Thomson renderers use (fomo-nearestneighbour.cpp:16-26,
// 100, 181; fomo-thomson.cpp:17-27, 209, 310).  Boost is not installed here and
// its version is not pinned by the reference (configure.ac:102 asks for >=1.54).
//
// What is restated, from Boost.Geometry's published semantics:
//  * model::point<float,3,cartesian>: three float coordinates; the constructor
//    takes the coordinate type, so double arguments are rounded to float at
//    the call site (this is how the reference's FP64 targets become FP32).
//  * index::within(box) on a point value: strictly inside in every dimension,
//    min < v && v < max (Boost's point-in-box "within" strategy; "covered_by"
//    would be <=).
//  * index::nearest(pt, k): the k values with the smallest comparable distance,
//    i.e. the squared Pythagorean distance computed in the promoted calculation
//    type (double for float coordinates) in the order Boost's
//    compute_pythagoras recursion uses: d_z*d_z + (d_y*d_y + (d_x*d_x + 0)),
//    with d = double(c1) - double(c2).
//  * rtree<value, quadratic<16>>: only the query result matters; the packing
//    algorithm changes traversal order and so, in Boost, which of several
//    exactly equidistant values is reported.  This shim scans every value and
//    breaks exact ties by insertion order (the lowest index), and returns the k
//    results sorted by distance.
// The scan is O(N) per query: the shim is for small fixture-sized cases only.
#ifndef FOMO_REFSHIM_BOOST_GEOMETRY_HPP
#define FOMO_REFSHIM_BOOST_GEOMETRY_HPP

#include <algorithm>
#include <cstddef>
#include <iostream>  // real Boost.Geometry headers pull in <iostream>
#include <utility>
#include <vector>

namespace boost {
namespace geometry {
namespace cs {
struct cartesian {};
}  // namespace cs

namespace model {
template <typename CoordinateType, std::size_t DimensionCount, typename CoordinateSystem>
class point {
 public:
  point() {
    for (std::size_t d = 0; d < DimensionCount; ++d) c_[d] = CoordinateType();
  }
  point(CoordinateType const& v0, CoordinateType const& v1 = CoordinateType(),
        CoordinateType const& v2 = CoordinateType()) {
    CoordinateType v[3] = {v0, v1, v2};
    for (std::size_t d = 0; d < DimensionCount; ++d) c_[d] = v[d];
  }
  CoordinateType get(std::size_t d) const { return c_[d]; }
  static constexpr std::size_t dimension = DimensionCount;

 private:
  CoordinateType c_[DimensionCount];
};

template <typename Point>
class box {
 public:
  box() {}
  box(Point const& min_corner, Point const& max_corner) : lo_(min_corner), hi_(max_corner) {}
  Point const& min_corner() const { return lo_; }
  Point const& max_corner() const { return hi_; }

 private:
  Point lo_, hi_;
};
}  // namespace model

namespace index {
template <std::size_t MaxElements, std::size_t MinElements = (MaxElements * 3) / 10>
struct quadratic {};

namespace detail {
template <typename Point>
struct nearest_pred {
  Point pt;
  unsigned k;
};
template <typename Box>
struct within_pred {
  Box box;
};
template <typename Point, typename Box>
struct nearest_within_pred {
  nearest_pred<Point> nearest;
  within_pred<Box> within;
};

// Boost.Geometry comparable (squared) Pythagorean distance, promoted to double.
template <typename P1, typename P2>
inline double comparable_distance(P1 const& p1, P2 const& p2) {
  double sum = 0.0;
  for (std::size_t d = 0; d < P1::dimension; ++d) {
    double const c1 = static_cast<double>(p1.get(d));
    double const c2 = static_cast<double>(p2.get(d));
    double const diff = c1 - c2;
    double const sq = diff * diff;
    sum = sq + sum;  // d_x^2 first, then d_y^2 + (..), then d_z^2 + (..)
  }
  return sum;
}

template <typename Point, typename Box>
inline nearest_within_pred<Point, Box> operator&&(nearest_pred<Point> const& n, within_pred<Box> const& w) {
  return nearest_within_pred<Point, Box>{n, w};
}

template <typename P, typename B>
inline bool strictly_within(P const& p, B const& b) {
  for (std::size_t d = 0; d < P::dimension; ++d) {
    if (!(b.min_corner().get(d) < p.get(d) && p.get(d) < b.max_corner().get(d))) return false;
  }
  return true;
}
}  // namespace detail

template <typename Point>
inline detail::nearest_pred<Point> nearest(Point const& pt, unsigned k) {
  return detail::nearest_pred<Point>{pt, k};
}
template <typename Box>
inline detail::within_pred<Box> within(Box const& b) {
  return detail::within_pred<Box>{b};
}

template <typename Value, typename Parameters>
class rtree {
 public:
  template <typename Iterator>
  rtree(Iterator first, Iterator last) : values_(first, last) {}

  template <typename Point, typename Box, typename OutIter>
  std::size_t query(detail::nearest_within_pred<Point, Box> const& pred, OutIter out) const {
    std::vector<std::pair<double, std::size_t> > hits;
    for (std::size_t i = 0; i < values_.size(); ++i) {
      if (!detail::strictly_within(values_[i].first, pred.within.box)) continue;
      hits.push_back(std::make_pair(detail::comparable_distance(pred.nearest.pt, values_[i].first), i));
    }
    std::size_t k = std::min<std::size_t>(pred.nearest.k, hits.size());
    std::partial_sort(hits.begin(), hits.begin() + k, hits.end());
    for (std::size_t r = 0; r < k; ++r) *out++ = values_[hits[r].second];
    return k;
  }

 private:
  std::vector<Value> values_;
};
}  // namespace index
}  // namespace geometry
}  // namespace boost

#endif
