// Internal glue shared by the translation units that implement include/qt_rgf.h:
// error-return macros and accessors for the opaque context.
#pragma once
#include <cuda_runtime.h>

#include "../../include/qt_rgf.h"
#include "qt_common.cuh"

#define QT_FAIL(code, msg)                             \
  do {                                                 \
    qt_set_last_error((msg), __FILE__, __LINE__);      \
    return (code);                                     \
  } while (0)

#define QT_TRY(expr)                                   \
  do {                                                 \
    qt_status _s = (expr);                             \
    if (_s != QT_OK) return _s;                        \
  } while (0)

namespace qt {
int ctx_device(const qt_ctx* c);
cudaStream_t ctx_stream(const qt_ctx* c);
}  // namespace qt
