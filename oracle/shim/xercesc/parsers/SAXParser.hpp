// Minimal declaration standing in for Xerces-C's SAXParser (see HandlerBase.hpp).
#ifndef ORACLE_SHIM_SAXPARSER_HPP
#define ORACLE_SHIM_SAXPARSER_HPP
class SAXParser {
 public:
  enum ValSchemes { Val_Never, Val_Always, Val_Auto };
};
#endif
