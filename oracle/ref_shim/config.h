/*
 * Stand-in for the header that the reference's CMake step generates from
 * config.h.in (config.h.in:1-25).  Test infrastructure only: it lets the
 * reference's unmodified host sources compile for the oracle build.
 */
#define _CRT_SECURE_NO_WARNINGS
#define HAVE_DIRENT_H
#include <dirent.h>
#include <cstring>
#include <stdexcept>
#include <string>

#define MAX_PLATFORM_NUM 10
#define MAX_DEVICE_NUM 1000

#define CAS_OFFINDER_VERSION "3.0.0"
#define CAS_OFFINDER_HOMEPAGE_URL "http://github.com/snugel/cas-offinder"
