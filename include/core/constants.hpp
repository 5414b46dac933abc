// constants.hpp — edges per read() call of the loader and vertices per CPBT page
// (the reference's core/constants.hpp:20-21; the page size enters the partition boundaries).
#ifndef EG_CORE_CONSTANTS_HPP
#define EG_CORE_CONSTANTS_HPP

#define CHUNKSIZE (1 << 20)
#define PAGESIZE (1 << 12)

#endif
