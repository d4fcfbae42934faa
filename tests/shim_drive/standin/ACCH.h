/* Stand-in declarations of MURaM's host/device copy points (include/ACCH.h). */
#pragma once
#include <cstddef>
namespace ACCH {
void UpdateCPU(void* ptr, std::size_t bytes);
void UpdateGPU(void* ptr, std::size_t bytes);
}  // namespace ACCH
