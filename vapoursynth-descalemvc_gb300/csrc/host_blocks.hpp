// Registry of host memory blocks registered with CUDA for direct transfers
// (the reference's direct block registration, src/host_blocks.cpp and
// include/dsmvc/host_blocks.hpp, for its CUDA domain).
//
// A frame host (a plugin's frame pool) reports the blocks its planes live in
// before each transfer (note_use).  A block is registered (page-locked with
// cudaHostRegister) on its second use, while its owner's registered bytes
// stay within the owner's cap; from then on the executor's copies from and
// to planes inside it are plain DMA instead of staged pageable copies.  A
// block already page-locked by someone else counts as registered and is
// never unregistered here.  The host releases a block before returning it
// to the system (release_block) or all of an owner's blocks at once
// (drop_owner).  Registration runs outside the registry's lock; a release
// that overlaps a registration in progress waits for it.
#pragma once

#include <cstddef>
#include <cstdint>

namespace dsmvc_gb {

struct HostBlockStats {
    std::uint64_t registrations = 0;    // blocks registered (ours or foreign)
    std::uint64_t failures = 0;         // registrations that failed
    std::uint64_t cap_refusals = 0;     // second uses refused by the owner's cap
    std::uint64_t hits = 0;             // covered() inside a registered block
    std::uint64_t misses = 0;           // covered() outside
    std::uint64_t released = 0;         // blocks we unregistered
    std::uint64_t registered_bytes = 0; // currently registered by us
    std::uint64_t peak_bytes = 0;
};

// Outcome of registering one block.
enum class BlockRegistration : int { failed = -1, owned = 0, foreign = 1 };

// The registration calls (CUDA by default; tests install fakes).
struct BlockRegistrar {
    BlockRegistration (*register_block)(void *base, std::size_t size) = nullptr;
    void (*unregister_block)(void *base, std::size_t size) = nullptr;
};

namespace host_blocks {

// Bytes one owner may keep registered (0: none, the default).
void set_limit(const void *owner, std::size_t bytes);
// Frame data inside [base, base + size) is about to be transferred.
void note_use(const void *owner, void *base, std::size_t size);
// [pointer, pointer + bytes) lies inside a registered block.
[[nodiscard]] bool covered(const void *pointer, std::size_t bytes);
// The block [base, base + size) is about to be freed.
void release_block(void *base, std::size_t size);
// Unregisters every block of `owner` and forgets the owner.
void drop_owner(const void *owner);
[[nodiscard]] HostBlockStats stats();
// Replaces the registration calls (everything registered is released first);
// a registrar with null calls restores CUDA's.
void set_registrar(const BlockRegistrar &registrar);
// CUDA's registration of one block, outside the registry (for a frame host
// that keeps its own).
[[nodiscard]] BlockRegistration cuda_register(void *base, std::size_t size);
void cuda_unregister(void *base, std::size_t size);

} // namespace host_blocks
} // namespace dsmvc_gb
