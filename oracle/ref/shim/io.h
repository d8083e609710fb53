/* io.h is a Windows header; the reference includes it on non-Apple systems
 * (MCRenderer.h:3-7, ConfigManager.h:3-9) and renames access to _access. */
#pragma once
#include <unistd.h>
static inline int _access(const char* path, int mode) { return access(path, mode); }
