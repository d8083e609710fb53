/* Force-included into every reference translation unit of the oracle build: headers
 * and std:: names the reference relies on implicitly (MSVC/libc++ provide them). */
#pragma once
#ifdef __cplusplus
#include <cstring>
#include <cmath>
#include <cstdlib>
namespace std {
using ::fabsf;
using ::powf;
}
#endif
