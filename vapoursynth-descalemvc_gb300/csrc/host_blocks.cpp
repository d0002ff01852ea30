// Host block registry (host_blocks.hpp).
#include "host_blocks.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <condition_variable>
#include <map>
#include <mutex>
#include <unordered_map>

namespace dsmvc_gb {
namespace host_blocks {

BlockRegistration cuda_register(void *base, std::size_t size) {
    const cudaError_t e = cudaHostRegister(base, size, cudaHostRegisterPortable);
    if (e == cudaSuccess) return BlockRegistration::owned;
    cudaGetLastError();   // the failed call leaves no sticky error behind
    return e == cudaErrorHostMemoryAlreadyRegistered ? BlockRegistration::foreign : BlockRegistration::failed;
}

void cuda_unregister(void *base, std::size_t) {
    if (cudaHostUnregister(base) != cudaSuccess) cudaGetLastError();
}

} // namespace host_blocks

namespace {

using host_blocks::cuda_register;
using host_blocks::cuda_unregister;

enum class State { seen, registering, registered, failed };

struct Block {
    std::size_t size = 0;
    const void *owner = nullptr;
    int uses = 0;
    State state = State::seen;
    bool owned = false;   // registered by us (unregistered on release)
};

struct Owner {
    std::size_t limit = 0;
    std::size_t used = 0;   // bytes registered or being registered for the owner
};

struct Registry {
    std::mutex mutex;
    std::condition_variable changed;
    std::map<std::uintptr_t, Block> blocks;   // by base address
    std::unordered_map<const void *, Owner> owners;
    BlockRegistrar registrar{cuda_register, cuda_unregister};
    HostBlockStats stats;
};

// Never destroyed: a frame pool may release blocks during static destruction.
Registry &registry() {
    static auto *r = new Registry;
    return *r;
}

using Lock = std::unique_lock<std::mutex>;

// Waits (lock held) until no registration matching `busy` is in progress.
template <class Pred> void wait_until_idle(Registry &r, Lock &lock, Pred busy) {
    r.changed.wait(lock, [&] {
        return std::none_of(r.blocks.begin(), r.blocks.end(), [&](const auto &kv) {
            return kv.second.state == State::registering && busy(kv.first, kv.second);
        });
    });
}

// Forgets a block (lock held, not being registered), unregistering it if
// it is ours.
void forget(Registry &r, std::map<std::uintptr_t, Block>::iterator it) {
    Block &b = it->second;
    if (b.state == State::registered && b.owned) {
        r.registrar.unregister_block(reinterpret_cast<void *>(it->first), b.size);
        Owner &o = r.owners[b.owner];
        o.used -= std::min(o.used, b.size);
        r.stats.registered_bytes -= std::min<std::uint64_t>(r.stats.registered_bytes, b.size);
        ++r.stats.released;
    }
    r.blocks.erase(it);
}

} // namespace

namespace host_blocks {

void set_limit(const void *owner, std::size_t bytes) {
    auto &r = registry();
    const std::scoped_lock lock(r.mutex);
    r.owners[owner].limit = bytes;
}

void note_use(const void *owner, void *base, std::size_t size) {
    if (!base || size == 0) return;
    auto &r = registry();
    Lock lock(r.mutex);
    const auto key = reinterpret_cast<std::uintptr_t>(base);
    auto it = r.blocks.find(key);
    if (it != r.blocks.end() && (it->second.owner != owner || it->second.size != size)) {
        // The address now holds another block: forget the old one.
        wait_until_idle(r, lock, [key](std::uintptr_t k, const Block &) { return k == key; });
        it = r.blocks.find(key);
        if (it != r.blocks.end()) forget(r, it);
        it = r.blocks.end();
    }
    if (it == r.blocks.end()) it = r.blocks.emplace(key, Block{size, owner}).first;
    Block &b = it->second;
    if (b.state != State::seen || ++b.uses < 2) return;
    Owner &o = r.owners[owner];
    if (o.limit == 0 || o.used + size > o.limit) {
        --b.uses;   // tried again on the next use, when there may be room
        ++r.stats.cap_refusals;
        return;
    }
    o.used += size;
    b.state = State::registering;
    const BlockRegistrar registrar = r.registrar;
    lock.unlock();
    const BlockRegistration outcome = registrar.register_block(base, size);
    lock.lock();
    // Still present: nothing erases a block while it is being registered.
    Block &done = r.blocks.at(key);
    Owner &owner_bytes = r.owners[owner];
    if (outcome == BlockRegistration::failed) {
        done.state = State::failed;
        owner_bytes.used -= std::min(owner_bytes.used, size);
        ++r.stats.failures;
    } else {
        done.state = State::registered;
        done.owned = outcome == BlockRegistration::owned;
        ++r.stats.registrations;
        if (done.owned) {
            r.stats.registered_bytes += size;
            r.stats.peak_bytes = std::max(r.stats.peak_bytes, r.stats.registered_bytes);
        } else {
            owner_bytes.used -= std::min(owner_bytes.used, size);
        }
    }
    lock.unlock();
    r.changed.notify_all();
}

bool covered(const void *pointer, std::size_t bytes) {
    auto &r = registry();
    const std::scoped_lock lock(r.mutex);
    const auto p = reinterpret_cast<std::uintptr_t>(pointer);
    auto it = r.blocks.upper_bound(p);
    bool hit = false;
    if (it != r.blocks.begin()) {
        --it;
        hit = it->second.state == State::registered && p + bytes <= it->first + it->second.size;
    }
    ++(hit ? r.stats.hits : r.stats.misses);
    return hit;
}

void release_block(void *base, std::size_t size) {
    if (!base || size == 0) return;
    auto &r = registry();
    Lock lock(r.mutex);
    const auto lo = reinterpret_cast<std::uintptr_t>(base), hi = lo + size;
    auto overlaps = [lo, hi](std::uintptr_t k, const Block &b) { return k < hi && k + b.size > lo; };
    wait_until_idle(r, lock, overlaps);
    for (auto it = r.blocks.begin(); it != r.blocks.end();) {
        auto next = std::next(it);
        if (overlaps(it->first, it->second)) forget(r, it);
        it = next;
    }
}

void drop_owner(const void *owner) {
    auto &r = registry();
    Lock lock(r.mutex);
    auto mine = [owner](std::uintptr_t, const Block &b) { return b.owner == owner; };
    wait_until_idle(r, lock, mine);
    for (auto it = r.blocks.begin(); it != r.blocks.end();) {
        auto next = std::next(it);
        if (it->second.owner == owner) forget(r, it);
        it = next;
    }
    r.owners.erase(owner);
}

HostBlockStats stats() {
    auto &r = registry();
    const std::scoped_lock lock(r.mutex);
    return r.stats;
}

void set_registrar(const BlockRegistrar &registrar) {
    auto &r = registry();
    Lock lock(r.mutex);
    wait_until_idle(r, lock, [](std::uintptr_t, const Block &) { return true; });
    while (!r.blocks.empty()) forget(r, r.blocks.begin());
    for (auto &[owner, o] : r.owners) o.used = 0;
    r.registrar = registrar.register_block && registrar.unregister_block ? registrar
                                                                         : BlockRegistrar{cuda_register, cuda_unregister};
}

} // namespace host_blocks
} // namespace dsmvc_gb
