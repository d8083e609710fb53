/* Case alias for a case-sensitive filesystem: the reference includes "scene.h" but ships "Scene.h". */
#pragma once
#include "Scene.h"
