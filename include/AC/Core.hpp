/*
 * Umbrella header of the GB300 backend's C++ interface, in place of the
 * reference's AC/Core.hpp: ac::core::Image, the model descriptors and
 * ac::core::Processor.  Link with libac_gb300.so.
 */
#ifndef AC_GB300_CXX_CORE_HPP
#define AC_GB300_CXX_CORE_HPP

#include "AC/Core/Image.hpp"
#include "AC/Core/Model.hpp"
#include "AC/Core/Processor.hpp"

#endif
