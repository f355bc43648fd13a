/*
 * Stand-in for the header that the reference's CMake step generates
 * (CMakeModules/CopyKernels.cmake:1-5), which embeds cas-offinder.cl as a
 * string.  The oracle's host emulator compiles cas-offinder.cl as C++ and binds
 * the kernels by name, so the source string is not needed.  Test infrastructure.
 */
static const char* program_src = "/* kernels are compiled natively by the oracle's host emulator */";
