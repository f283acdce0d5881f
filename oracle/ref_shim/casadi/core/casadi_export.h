/* Stand-in for the export-macro header CMake generates for libcasadi: public classes get
 * default visibility, as in the reference's shared-library build. */
#ifndef CASADI_EXPORT_H_SHIM
#define CASADI_EXPORT_H_SHIM
#define CASADI_EXPORT __attribute__((visibility("default")))
#define CASADI_NO_EXPORT __attribute__((visibility("hidden")))
#define CASADI_DEPRECATED __attribute__((__deprecated__))
#endif
