// Stand-in for the reference's include/vulkan/vk.hpp when its shared GLSL
// headers are compiled in their C++ mode for the oracle's reference build:
// those headers only need the VkDeviceAddress type from it (the real header
// pulls in the Vulkan SDK, which is absent here).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstdint>
typedef std::uint64_t VkDeviceAddress;
