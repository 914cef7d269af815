/* TEST INFRASTRUCTURE: stands in for the header the reference's CMake
 * configuration writes from src/rschol/config.h.in.  Only the zlib switch
 * is set (zlib is present); no CBLAS include-file name is needed because
 * the shim directory provides cblas.h. */
#ifndef CONFIG_H
#define CONFIG_H
#define HAS_ZLIB
#endif
