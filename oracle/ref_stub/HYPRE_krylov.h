/* Single-rank stand-in: see vfs_ref_stub.h. */
#include "vfs_ref_stub.h"
