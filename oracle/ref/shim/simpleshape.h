/* Case alias for a case-sensitive filesystem: the reference includes "simpleshape.h" but ships "SimpleShape.h". */
#pragma once
#include "SimpleShape.h"
