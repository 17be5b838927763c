// Header shim: see boost/iostreams/filtering_streambuf.hpp.
#include <boost/iostreams/filtering_streambuf.hpp>
