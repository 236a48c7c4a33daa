/* stand-in: everything is in nanobind.h (parity-check builds only) */
#include "../nanobind.h"
