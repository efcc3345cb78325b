/* Forwards to the oracle's GSL-API subset (not GSL). */
#include "../gslsub.h"
