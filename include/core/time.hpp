// time.hpp — wall-clock seconds (get_time of the reference, core/time.hpp:22-26)
#ifndef EG_CORE_TIME_HPP
#define EG_CORE_TIME_HPP

#include <chrono>

inline double get_time() {
    return std::chrono::duration<double>(std::chrono::system_clock::now().time_since_epoch()).count();
}

#endif
