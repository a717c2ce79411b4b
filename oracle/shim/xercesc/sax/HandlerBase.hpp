// Minimal declarations standing in for Xerces-C's SAX handler base class.
// The reference's ShapeParser.h includes this header; the oracle build never
// parses XML (meshes are read by oracle/ref_harness.cpp), so only the names
// that ShapeParser.h mentions are declared here.
#ifndef ORACLE_SHIM_HANDLERBASE_HPP
#define ORACLE_SHIM_HANDLERBASE_HPP
#define XERCES_CPP_NAMESPACE_USE
typedef unsigned short XMLCh;
class AttributeList {};
class HandlerBase {
 public:
  virtual ~HandlerBase() {}
};
#endif
