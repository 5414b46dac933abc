// atomic.hpp — cas / write_min / write_add with the reference's semantics (core/atomic.hpp:25-52):
// cas swaps iff the value equals old_val; write_min lowers *ptr to val and reports whether this
// call did it; write_add adds atomically (also for floating point).
#ifndef EG_CORE_ATOMIC_HPP
#define EG_CORE_ATOMIC_HPP

#include <string.h>

template <class T>
inline bool cas(T* ptr, T old_val, T new_val) {
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "cas needs a 4- or 8-byte type");
    return __atomic_compare_exchange(ptr, &old_val, &new_val, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
}

template <class T>
inline bool write_min(T* ptr, T val) {
    T cur;
    __atomic_load(ptr, &cur, __ATOMIC_RELAXED);
    while (val < cur) {
        if (__atomic_compare_exchange(ptr, &cur, &val, false, __ATOMIC_SEQ_CST, __ATOMIC_RELAXED)) return true;
    }
    return false;
}

template <class T>
inline void write_add(T* ptr, T val) {
    T cur;
    __atomic_load(ptr, &cur, __ATOMIC_RELAXED);
    T next = cur + val;
    while (!__atomic_compare_exchange(ptr, &cur, &next, false, __ATOMIC_SEQ_CST, __ATOMIC_RELAXED)) next = cur + val;
}

#endif
