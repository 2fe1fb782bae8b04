// Link stubs for the out-of-tree build of the UG reference (test oracle only).
// UG's binary file I/O (low/bio.cc, ui/fieldio.cc) needs the XDR headers
// (rpc/rpc.h), which are not installed; the oracle never saves or loads
// multigrids, so these entry points only report failure.
#include <config.h>
#include <cstdio>
#include "ugtypes.h"
#include "namespace.h"

namespace UG {
int Bio_Read_mint(int, int *) { return 1; }
int Bio_Write_mint(int, int *) { return 1; }
int Bio_Write_string(const char *) { return 1; }
int Bio_Read_string(char *) { return 1; }
int Bio_Write_mdouble(int, double *) { return 1; }
int Bio_Read_mdouble(int, double *) { return 1; }
int Bio_Initialize(FILE *, int, char) { return 1; }
int Bio_Jump_To() { return 1; }
int Bio_Jump_From() { return 1; }
int Bio_Jump(int) { return 1; }
#ifdef _2
namespace D2 { int InitFieldIO() { return 0; } }
#else
namespace D3 { int InitFieldIO() { return 0; } }
#endif
}  // namespace UG
