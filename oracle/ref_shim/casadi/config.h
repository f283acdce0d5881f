/* Stand-in for the configure-time header of libcasadi (version of the reference). */
#ifndef CASADI_CONFIG_H_SHIM
#define CASADI_CONFIG_H_SHIM
#define CASADI_MAJOR_VERSION 3
#define CASADI_MINOR_VERSION 7
#define CASADI_PATCH_VERSION 2
#define CASADI_IS_RELEASE 0
#define CASADI_VERSION_STRING "3.7.2"
#endif
