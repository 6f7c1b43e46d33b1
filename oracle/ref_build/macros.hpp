// Configuration header for compiling the reference solver as a CPU oracle.
// The reference generates this header from a CMake template; these are the
// same macro names with the values that template produces for v0.10.0
// (reference CMakeLists.txt sets the version, include/macros.hpp.in holds the
// numeric constants).  Release configuration: assertions compiled out.
#ifndef MACROSHEADERDEF
#define MACROSHEADERDEF

#define EPS 1.0e-30
#define ROOTP 0
#define DEFAULT_WALL_DIST 1.0e10
#define WALL_DIST_NEG_TOL -1.0e-10
#define MAJORVERSION 0
#define MINORVERSION 10
#define PATCHNUMBER 0

#ifndef NDEBUG
#define MSG_ASSERT(expr, msg) \
  AssertWithMessage(#expr, expr, __FILE__, __LINE__, msg)
#else
#define MSG_ASSERT(expr, msg) ;
#endif

void AssertWithMessage(const char *exprStr, bool expr, const char *file,
                       int line, const char *msg);

#endif
