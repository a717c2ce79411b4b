// Stand-in for Xerces-C's xercesc/util/OutOfMemoryException.hpp: see oracle/shim/xercesc/shim_core.hpp.
#include "../shim_core.hpp"
