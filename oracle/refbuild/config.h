/* config.h -- the build configuration the reference's autotools would
 * generate, fixed for the oracle's single-process FP64 build (TEST
 * INFRASTRUCTURE).  No OpenMP, no debug output. */
#define PNFFT_ENABLE_DEBUG 0
#define PACKAGE_VERSION "1.0.7-alpha (oracle reference build)"
#define HAVE_MALLOC_H 1
