// Stand-in for the two Win32 calls the SPHNJ reference makes (main.cu:32,
// output.cu:260 and friends), so its sources build on Linux for the
// reference-build harness.  Not part of libsphnj.
#ifndef SPHNJ_WINDOWS_SHIM_H
#define SPHNJ_WINDOWS_SHIM_H
#include <sys/stat.h>
#include <unistd.h>
inline void Sleep(unsigned ms) { usleep(ms * 1000u); }
inline int CreateDirectory(const char *path, void *) { return mkdir(path, 0755) == 0; }
#endif
