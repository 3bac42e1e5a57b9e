/* Minimal GSL error codes (test oracle only). */
#ifndef ENB_REFSHIM_GSL_ERRNO_H
#define ENB_REFSHIM_GSL_ERRNO_H
enum { GSL_SUCCESS = 0, GSL_FAILURE = -1, GSL_CONTINUE = -2, GSL_EINVAL = 4, GSL_EBADFUNC = 9, GSL_ENOPROG = 27 };
#endif
