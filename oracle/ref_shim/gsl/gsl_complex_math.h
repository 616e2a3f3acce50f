/* Empty stand-in (see gsl_blas.h). */
#pragma once
