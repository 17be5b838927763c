/*
 * Header shim for building the reference's FoMo-C sources in the test harness
 * (oracle/_ref).  GSL is not installed here; the reference only uses three
 * physical constants from this header (fomo-CHIANTI.cpp:17-19,
 * fomo-nearestneighbour.cpp:28, fomo-rendercube.cpp:7, fomo-thomson.cpp:29).
 *
 * Values: the MKSA constants shipped in GSL's gsl_const_mksa.h (GSL 1.x/2.x):
 * c is exact by definition; k_B is the CODATA-2006 value and m_p the CODATA-1998
 * value that GSL ships.  The same numbers are used by the oracle restatement
 * (oracle/fomo_oracle.h) and by the GPU library (fomo_gb300/csrc/fomo_consts.h).
 */
#ifndef FOMO_REFSHIM_GSL_CONST_MKSA_H
#define FOMO_REFSHIM_GSL_CONST_MKSA_H
#define GSL_CONST_MKSA_SPEED_OF_LIGHT (2.99792458e8)
#define GSL_CONST_MKSA_BOLTZMANN (1.3806504e-23)
#define GSL_CONST_MKSA_MASS_PROTON (1.67262158e-27)
#endif
