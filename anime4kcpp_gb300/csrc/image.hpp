// The backend's host image is the public ac::core::Image
// (include/AC/Core/Image.hpp); the internal code names it acgb::Image.
#pragma once

#include "AC/Core/Image.hpp"

namespace acgb {
using Image = ac::core::Image;
}  // namespace acgb
