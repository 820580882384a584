/*
 * Error codes of the C ABI.
 * Same values as the reference binding (binding/c/include/AC/Error.h:4-9),
 * so callers that test for AC_ERROR(AC_EPROCESSOR) keep working unchanged.
 */
#ifndef AC_GB300_ERROR_H
#define AC_GB300_ERROR_H

#define AC_SUCCESS 0
#define AC_ERROR(e) (-(e))

#define AC_EIO          5
#define AC_EINVAL      22
#define AC_EPROCESSOR 256

#endif
