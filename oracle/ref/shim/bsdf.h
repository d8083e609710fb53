/* Case alias for a case-sensitive filesystem: the reference includes "bsdf.h" but ships "BSDF.h". */
#pragma once
#include "BSDF.h"
