// filesystem.hpp — file_exists / file_size (the reference's core/filesystem.hpp:27-36)
#ifndef EG_CORE_FILESYSTEM_HPP
#define EG_CORE_FILESYSTEM_HPP

#include <sys/stat.h>

#include <string>

inline bool file_exists(std::string filename) {
    struct stat st;
    return stat(filename.c_str(), &st) == 0;
}

inline long file_size(std::string filename) {
    struct stat st;
    if (stat(filename.c_str(), &st) != 0) return -1;
    return (long)st.st_size;
}

#endif
