/*
 * Processor handles of the C ABI.
 *
 * Drop-in replacement for the reference binding's processor API
 * (binding/c/include/AC/Core/Processor.h:15-36, implemented in
 * binding/c/src/Binding.cpp:163-247).  A processor created with type "cuda"
 * or "auto" runs the whole upscaling path -- RGB->YUV split, luma CNN x2
 * passes, chroma resize, YUV->RGB merge -- on one GB300 GPU.  There is no
 * CPU fallback: types "cpu" and "opencl" yield a processor whose
 * ac_processor_ok() is AC_ERROR(AC_EPROCESSOR) and whose ac_processor_error()
 * says why.
 *
 * Models (the reference's model strings, parsed like
 * core/src/processor/Processor.cpp:26-187):
 *   "acnet-legacy-gan", "acnet-legacy-hdn0".."-hdn3"      ACNetLegacy
 *   "acnet-f8b4|b8|b18[-hdn][-box][-box-hdn]"             ACNet<8>
 *   "artcnn-c4f16|c4f32[-dn|-ds]"                         ArtCNN<16/32>
 *   "fsrcnnx-f8|f16[-dp]"                                 FSRCNNX<8/16>
 *   "arnet-[hdn-][box-]b8|b16|b32|b64"                    ARNet<8>
 * ACNetLegacy, ACNet<8>, ArtCNN and FSRCNNX run the reference's trained
 * parameters; ARNet runs its exact topology with seeded synthetic parameters
 * (the reference's trained ARNet parameters are not in its source tree).
 */
#ifndef AC_GB300_PROCESSOR_H
#define AC_GB300_PROCESSOR_H

#include <stdint.h>

#include "ac_image.h"

/* Processor.h:8-13. */
enum ACProcessorType
{
    AC_PROCESSOR_CPU    = 0,
    AC_PROCESSOR_OPENCL = 1,
    AC_PROCESSOR_CUDA   = 2
};

/* Processor.h:15-21: same field order and types; type/model are borrowed
 * and read only by ac_processor_create. */
typedef struct ACProcessor
{
    int device;
    const char* type;
    const char* model;
    struct ACProcessorHandle* hptr;
} ACProcessor;

/* Replaces Processor.h:23 / Binding.cpp:163-168. */
AC_C_API ACProcessor* ac_processor_alloc(void);
/* Replaces Processor.h:24 / Binding.cpp:169-175. */
AC_C_API void ac_processor_free(ACProcessor** processor);
/* Replaces Processor.h:25 / Binding.cpp:176-185. */
AC_C_API int ac_processor_ref(const ACProcessor* src, ACProcessor* dst);
/* Replaces Processor.h:26 / Binding.cpp:186-191. */
AC_C_API void ac_processor_unref(ACProcessor* processor);
/* Replaces Processor.h:27 / Binding.cpp:192-198: returns ac_processor_ok(). */
AC_C_API int ac_processor_create(ACProcessor* processor);
/* Replaces Processor.h:28 / Binding.cpp:199-205: Processor::process(src, dst, factor)
 * semantics of core/src/processor/Processor.cpp:199-276 (a non-empty dst is
 * taken as preallocated with the right shape), then mirrors dst's fields. */
AC_C_API int ac_processor_process(ACProcessor* processor, const ACImage* src, ACImage* dst, double factor);
/* Replaces Processor.h:29 / Binding.cpp:206-210: per calling thread. */
AC_C_API int ac_processor_ok(const ACProcessor* processor);
/* Replaces Processor.h:30 / Binding.cpp:211-215: per calling thread. */
AC_C_API const char* ac_processor_error(const ACProcessor* processor);
/* Replaces Processor.h:31 / Binding.cpp:216-220: the device name. */
AC_C_API const char* ac_processor_name(const ACProcessor* processor);
/* Replaces Processor.h:32 / Binding.cpp:221-225: AC_PROCESSOR_CUDA. */
AC_C_API int ac_processor_type(const ACProcessor* processor);
/* Replaces Processor.h:33 / Binding.cpp:226-230: "CUDA". */
AC_C_API const char* ac_processor_type_name(const ACProcessor* processor);

/* Replaces Processor.h:35 / Binding.cpp:232-244. */
AC_C_API const char* ac_processor_info(int processor_type);
/* Replaces Processor.h:36 / Binding.cpp:245-247. */
AC_C_API const char* ac_processor_list_info(void);

#endif
