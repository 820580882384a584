/* Umbrella header, the counterpart of binding/c/include/AC/Core.h. */
#ifndef AC_GB300_CORE_H
#define AC_GB300_CORE_H

#include "ac_error.h"
#include "ac_image.h"
#include "ac_processor.h"

#endif
