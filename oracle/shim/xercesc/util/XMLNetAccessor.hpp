// Stand-in for Xerces-C's xercesc/util/XMLNetAccessor.hpp: see oracle/shim/xercesc/shim_core.hpp.
#include "../shim_core.hpp"
