/* Test-only stand-in for the CMake-generated GWATConfig.h of the reference,
 * for the oracle pin build (oracle/Makefile).  The share directory is unused
 * on the pinned path. */
#ifndef GWO_SHIM_GWATCONFIG_H
#define GWO_SHIM_GWATCONFIG_H
#define GWAT_VERSION_MAJOR 0
#define GWAT_VERSION_MINOR 0
#define GWAT_ROOT_DIRECTORY ""
#define GWAT_INSTALL_PREFIX ""
#define GWAT_SHARE_DIR ""
#endif
