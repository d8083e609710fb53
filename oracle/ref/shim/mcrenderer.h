/* Case alias for a case-sensitive filesystem: the reference includes "mcrenderer.h" but ships "MCRenderer.h". */
#pragma once
#include "MCRenderer.h"
