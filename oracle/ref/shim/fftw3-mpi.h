/* FFTW-MPI stand-in: the reference includes it but never calls into it on the sine path. */
#include "fftw3.h"
