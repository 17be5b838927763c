/* Stand-in for the autoconf-generated config.h the reference sources include
 * as "../config.h".  No optional feature (MPI, CGAL, TBB, VTK) is enabled. */
#ifndef FOMO_REFSHIM_CONFIG_H
#define FOMO_REFSHIM_CONFIG_H
#endif
