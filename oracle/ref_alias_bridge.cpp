// ref_alias_bridge.cpp -- the reference's own createAliasTable
// (src/misc.cpp:416-497, the Vose alias method over light power) compiled on
// the CPU.  misc.cpp includes Vulkan and does not build here, so the recipe in
// oracle/Makefile copies exactly that function, unchanged, out of the
// reference tree into oracle/_ref/alias/createAliasTable.inc; this bridge
// supplies the headers it needs (<queue>, <vector>, the shader structs of
// src/shaderIncludes.h) and a C entry point.
//
// TEST INFRASTRUCTURE ONLY.  Built into oracle/_ref/ from the reference
// sources where they lie; nothing here is shipped.
#include <cstdint>
#include <cstring>
#include <queue>
#include <vector>

#include "nvmath.h"
#include "shaderIncludes.h"

#include "createAliasTable.inc"

extern "C" {

// pl: n_pl pointLight records (32 B); tl: n_tl triLight records (80 B);
// out: one aliasTableColumn (16 B) per light.  Returns the column count.
int32_t ref_create_alias_table(const void *pl, int32_t n_pl, const void *tl, int32_t n_tl, void *out) {
    static_assert(sizeof(shader::pointLight) == 32 && sizeof(shader::triLight) == 80 &&
                      sizeof(shader::aliasTableColumn) == 16,
                  "reference layouts");
    std::vector<shader::pointLight> pts((size_t)(n_pl > 0 ? n_pl : 0));
    std::vector<shader::triLight> tris((size_t)(n_tl > 0 ? n_tl : 0));
    if (!pts.empty()) std::memcpy(pts.data(), pl, pts.size() * sizeof(shader::pointLight));
    if (!tris.empty()) std::memcpy(tris.data(), tl, tris.size() * sizeof(shader::triLight));
    const std::vector<shader::aliasTableColumn> cols = createAliasTable(pts, tris);
    std::memcpy(out, cols.data(), cols.size() * sizeof(shader::aliasTableColumn));
    return (int32_t)cols.size();
}

}  // extern "C"
