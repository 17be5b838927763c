// Header shim: everything the reference uses lives in boost/geometry.hpp.
#include <boost/geometry.hpp>
