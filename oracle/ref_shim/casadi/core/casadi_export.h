/* Stand-in for the export-macro header CMake generates for libcasadi: the harness links
 * the reference's header-only op semantics statically, so nothing is exported. */
#ifndef CASADI_EXPORT_H_SHIM
#define CASADI_EXPORT_H_SHIM
#define CASADI_EXPORT
#define CASADI_NO_EXPORT
#define CASADI_DEPRECATED
#endif
