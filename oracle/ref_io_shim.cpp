// C-ABI shim around the reference's own output writers, compiled by oracle/build_ref.sh together
// with the reference's unmodified src/util_io.cpp and its vendored VoxWriter into
// oracle/_ref/libref_io.so.  Test infrastructure only (it generates golden files; never the
// product).  It exposes:
//   ref_write_binvox -> write_binvox (src/util_io.cpp:202-246), writing <base>_<gx>.binvox
#include <cstdint>
#include <cstring>
#include <string>
#include "util_io.h"

static_assert(sizeof(voxinfo) == 64, "voxinfo layout");

extern "C" void ref_write_binvox(const uint32_t* table, const void* info64, const char* base) {
	alignas(voxinfo) unsigned char buf[sizeof(voxinfo)];
	std::memcpy(buf, info64, sizeof(voxinfo));
	const voxinfo& info = *reinterpret_cast<const voxinfo*>(buf);
	write_binvox(table, info, std::string(base));
	std::fflush(stdout);
}
