// Physical constants of FoMo-C's render path.
//  * c, k_B, m_p: the MKSA values GSL ships in gsl_const_mksa.h, which the
//    reference uses (fomo-c/src/fomo-CHIANTI.cpp:17-19, fomo-nearestneighbour.cpp:28).
//  * alpha = sqrt(2 pi)/2/sqrt(2 ln 2) rounded as in fomo-CHIANTI.cpp:16.
//  * 0.715 Mm per arcsec (fomo-c/src/FoMo-internal.h:4).
//  * Thomson: R_sun, limb darkening, electron radius, irradiance (fomo-thomson.cpp:31-34).
#pragma once

#define FOMO_SPEED_OF_LIGHT 2.99792458e8
#define FOMO_BOLTZMANN 1.3806504e-23
#define FOMO_MASS_PROTON 1.67262158e-27
#define FOMO_ALPHA 1.0645
#define FOMO_MM_PER_ARCSEC 0.715
#define FOMO_RSUN 695.7
#define FOMO_LIMB_U 0.58
#define FOMO_ELECTRON_RADIUS 2.8179e-13
#define FOMO_IRRADIANCE 2.8e10
#define FOMO_PI 3.14159265358979323846
