// Error handling of the extern "C" entry points: a tnad::Error thrown inside
// becomes its TNAD_ERR_* return code, with the message kept on the context.
#pragma once

#include <exception>

#include "tnad_internal.h"

#define API_BEGIN(c)                         \
  if (!(c)) return TNAD_ERR_ARG;             \
  try {                                      \
    TNAD_CK(cudaSetDevice((c)->device));
#define API_END(c)                           \
  }                                          \
  catch (const tnad::Error& e) {             \
    (c)->err = e.msg;                        \
    cudaStreamSynchronize((c)->stream);      \
    return e.code;                           \
  }                                          \
  catch (const std::exception& e) {          \
    (c)->err = e.what();                     \
    return TNAD_ERR_ARG;                     \
  }                                          \
  return TNAD_OK;
