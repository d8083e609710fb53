/* Case alias for a case-sensitive filesystem: the reference includes "sceneobject.h" but ships "SceneObject.h". */
#pragma once
#include "SceneObject.h"
