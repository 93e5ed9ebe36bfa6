// Status check shared by the reference-side shims: a failed library call
// throws std::runtime_error with the library's message (the reference itself
// has no error channel; its driver can catch this and call MPI_Abort).
#ifndef GB300_CHECK_HH
#define GB300_CHECK_HH

#include <stdexcept>
#include <string>

#include "lbm_gb300.h"

inline void gb300_check(lbm_status s, const char* what, const char* detail)
{
   if (s != LBM_OK)
      throw std::runtime_error(std::string(what) + ": " + lbm_status_string(s) + " (" + (detail ? detail : "") + ")");
}

#endif
