// Internal runtime services shared by the entry points.
#pragma once

#include <cstddef>
#include <mutex>

namespace sigma {

// Serialises the host-pointer entry points (they share cached buffers).
std::mutex& api_mutex();

// Multiprocessor count of the current device (0 when no device).
int device_sm_count();

// Grow-only device buffers of the current device, one per slot; freed by
// sigma_shutdown().  The caller holds api_mutex().
constexpr int kArenaSlots = 4;
enum ArenaSlot { kArenaGppInputs = 0, kArenaFfInputs = 1, kArenaBatched = 2, kArenaMisc = 3 };
int arena_get(int slot, size_t bytes, void** out);

void set_last_error_text(const char* text);

// Functions run by sigma_shutdown() before the arenas are freed (plan caches).
typedef void (*ShutdownHook)();
void register_shutdown_hook(ShutdownHook h);

}  // namespace sigma
