// Stand-in for Xerces-C's xercesc/util/TransService.hpp: see oracle/shim/xercesc/shim_core.hpp.
#include "../shim_core.hpp"
