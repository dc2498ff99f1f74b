// Stub for the reference's Vulkan memory wrapper (src/vma.h).
// TEST INFRASTRUCTURE ONLY: src/aabbTreeBuilder.h:25-51 declares an upload
// helper against this API; the stub lets that header parse without Vulkan.
// The helper is never called.
#pragma once
#include <cassert>
#include <cstdint>
#include <cstring>

namespace vk {
using DeviceSize = uint64_t;
enum class BufferUsageFlagBits : uint32_t { eStorageBuffer = 0x20 };
}  // namespace vk
enum { VMA_MEMORY_USAGE_CPU_TO_GPU = 3 };

namespace vma {
struct UniqueBuffer {
    void *ptr = nullptr;
    template <typename T> T *mapAs() { return static_cast<T *>(ptr); }
    void unmap() {}
    void flush() {}
};
class Allocator {
public:
    UniqueBuffer createBuffer(uint32_t, vk::BufferUsageFlagBits, int) { return UniqueBuffer{}; }
};
}  // namespace vma
