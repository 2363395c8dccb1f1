/* The host runtime of include/sofren2.h compiled once with exported symbols, so that the
 * shared library libsofren2_gb300.so offers the sft_* API to non-C callers (ctypes). */
#define SFT_IMPL
#define SFT_NO_DEBUG
#define SFT_FUNC __attribute__((visibility("default")))
#include "../../include/sofren2.h"
