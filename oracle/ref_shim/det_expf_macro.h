/* Forced include of the checker's second build of the reference's frame helpers:
 * their expf calls evaluate the Cody-Waite exp of det_expf.h, the one the frame
 * kernel and the oracle use, so that build agrees with both bit for bit.  The
 * math headers are read first, with expf undefined. */
#pragma once
#include <cmath>
#include <math.h>
#include "../det_expf.h"
#define expf(x) gca_det_expf(x)
