/*
 * Force-included into every reference translation unit of oracle/_ref -- TEST INFRASTRUCTURE
 * ONLY.  The reference was written for C++98, where a stream converts implicitly to void* and
 * so can be written to another stream (src/Printer.cpp:131 does that in an error message).
 * C++11 made the conversion explicit; this overload restores the C++98 output (the stream's
 * state as a pointer value) so the file compiles unchanged under a current compiler.
 */
#ifndef IMPEC_REFSHIM_CXX98_COMPAT_H
#define IMPEC_REFSHIM_CXX98_COMPAT_H
#ifdef __cplusplus
#include <fstream>
#include <ostream>
inline std::ostream& operator<<(std::ostream& os, const std::ofstream& f) {
    return os << (const void*)(f.fail() ? nullptr : &f);
}
#endif
#endif
