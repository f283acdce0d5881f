/* Stand-in for the configure-time header of libcasadi: the version of the reference and the
 * build facts casadi_meta.cpp reports. No configure step runs; this file replaces it. */
#ifndef CASADI_CONFIG_H_SHIM
#define CASADI_CONFIG_H_SHIM
#define CASADI_MAJOR_VERSION 3
#define CASADI_MINOR_VERSION 7
#define CASADI_PATCH_VERSION 2
#define CASADI_IS_RELEASE 0
#define CASADI_VERSION_STRING "3.7.2"
#define CASADI_GIT_REVISION ""
#define CASADI_GIT_DESCRIBE ""
#define CASADI_FEATURE_LIST ""
#define CASADI_BUILD_TYPE "Release"
#define CASADI_COMPILER_ID "GNU"
#define CASADI_COMPILER "g++"
#define CASADI_COMPILER_FLAGS "-O2"
#define CASADI_MODULES ""
#define CASADI_PLUGINS ""
#define CASADI_INSTALL_PREFIX ""
#define CASADI_SHARED_LIBRARY_PREFIX "lib"
#define CASADI_SHARED_LIBRARY_SUFFIX ".so"
#define CASADI_OBJECT_FILE_SUFFIX ".o"
#define CASADI_LAPACK_LIBRARIES ""
#endif
