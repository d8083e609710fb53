/* Case alias for a case-sensitive filesystem: the reference includes "SceneHeteroGeneousVolume.h" but ships "SceneHeterogeneousVolume.h". */
#pragma once
#include "SceneHeterogeneousVolume.h"
