// A small stand-in for the parts of Xerces-C that the reference's
// src/ShapeParser.cpp uses (Xerces is not installed here).  Test
// infrastructure of the oracle build only: it lets the reference's own X3D
// handler (ShapeParserHandler) run unmodified, so that the project's X3D
// reader can be checked against it on the reference's example files.
//
// What it provides: XMLCh strings (16-bit, ASCII content), XMLString's
// transcode / compareString / indexOf, an attribute list, the SAX handler base
// class, and a SAX parser that reads a file and reports start and end tags
// with their attributes (processing instructions, comments, DOCTYPE and text
// are skipped; the five predefined entities are decoded in attribute values).
#ifndef ORACLE_SHIM_XERCES_CORE_HPP
#define ORACLE_SHIM_XERCES_CORE_HPP

#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <utility>
#include <vector>

#define XERCES_CPP_NAMESPACE_USE

typedef unsigned short XMLCh;
typedef size_t XMLSize_t;

namespace oracle_shim {

inline size_t xlen(const XMLCh *s) {
  size_t n = 0;
  while (s && s[n]) n++;
  return n;
}

// Transcoded buffers are never freed (the reference does not release them).
// A char buffer ends in "\0 ": the reference's FaceIndex scanner walks to the
// next space after the last number of a string, and finds it just past the
// terminator.
inline XMLCh *to_xml(const std::string &s) {
  XMLCh *d = new XMLCh[s.size() + 1];
  for (size_t i = 0; i < s.size(); i++) d[i] = (unsigned char)s[i];
  d[s.size()] = 0;
  return d;
}

inline char *to_char(const XMLCh *s) {
  const size_t n = xlen(s);
  char *d = new char[n + 2];
  for (size_t i = 0; i < n; i++) d[i] = (char)s[i];
  d[n] = 0;
  d[n + 1] = ' ';
  return d;
}

}  // namespace oracle_shim

class XMLString {
 public:
  static XMLCh *transcode(const char *s) { return oracle_shim::to_xml(s ? s : ""); }
  static char *transcode(const XMLCh *s) { return oracle_shim::to_char(s); }
  static int compareString(const XMLCh *a, const XMLCh *b) {
    size_t i = 0;
    for (;; i++) {
      const XMLCh ca = a ? a[i] : 0, cb = b ? b[i] : 0;
      if (ca != cb) return (int)ca - (int)cb;
      if (!ca) return 0;
    }
  }
  static int indexOf(const char *s, const char ch, const XMLSize_t from) {
    const size_t n = strlen(s);
    for (size_t i = from; i < n; i++)
      if (s[i] == ch) return (int)i;
    return -1;
  }
  static void release(char **p) { delete[] *p; *p = nullptr; }
  static void release(XMLCh **p) { delete[] *p; *p = nullptr; }
};

class XMLException {
 public:
  explicit XMLException(const std::string &m = "XML error") : msg_(oracle_shim::to_xml(m)) {}
  const XMLCh *getMessage() const { return msg_; }

 private:
  XMLCh *msg_;
};

class NetAccessorException : public XMLException {
 public:
  using XMLException::XMLException;
};

class OutOfMemoryException {};

class XMLPlatformUtils {
 public:
  static void Initialize() {}
  static void Terminate() {}
};

class AttributeList {
 public:
  XMLSize_t getLength() const { return names_.size(); }
  const XMLCh *getName(XMLSize_t i) const { return i < names_.size() ? names_[i] : nullptr; }
  const XMLCh *getValue(XMLSize_t i) const { return i < values_.size() ? values_[i] : nullptr; }
  const XMLCh *getValue(const char *name) const {
    for (size_t i = 0; i < raw_.size(); i++)
      if (raw_[i].first == name) return values_[i];
    return nullptr;
  }
  void add(const std::string &n, const std::string &v) {
    raw_.push_back({n, v});
    names_.push_back(oracle_shim::to_xml(n));
    values_.push_back(oracle_shim::to_xml(v));
  }

 private:
  std::vector<std::pair<std::string, std::string>> raw_;
  std::vector<XMLCh *> names_, values_;
};

class HandlerBase {
 public:
  virtual ~HandlerBase() {}
  virtual void startElement(const XMLCh *const, AttributeList &) {}
  virtual void endElement(const XMLCh *const) {}
};

class SAXParser {
 public:
  enum ValSchemes { Val_Never, Val_Always, Val_Auto };
  void setValidationScheme(ValSchemes) {}
  void setDoNamespaces(bool) {}
  void setDoSchema(bool) {}
  void setValidationSchemaFullChecking(bool) {}
  void setDocumentHandler(HandlerBase *h) { handler_ = h; }

  void parse(const char *file) {
    FILE *f = fopen(file, "rb");
    if (!f) throw XMLException(std::string("cannot open ") + file);
    std::string doc;
    char buf[65536];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) doc.append(buf, n);
    fclose(f);
    size_t p = 0;
    while ((p = doc.find('<', p)) != std::string::npos) {
      if (doc.compare(p, 4, "<!--") == 0) {
        p = skip(doc, p, "-->");
      } else if (doc.compare(p, 2, "<?") == 0) {
        p = skip(doc, p, "?>");
      } else if (doc.compare(p, 2, "<!") == 0) {
        p = skip(doc, p, ">");
      } else if (doc.compare(p, 2, "</") == 0) {
        const size_t e = doc.find('>', p);
        if (e == std::string::npos) throw XMLException("unterminated end tag");
        std::string name = trim(doc.substr(p + 2, e - p - 2));
        XMLCh *x = oracle_shim::to_xml(name);
        if (handler_) handler_->endElement(x);
        p = e + 1;
      } else {
        p = start_tag(doc, p + 1);
      }
    }
  }

 private:
  static size_t skip(const std::string &d, size_t p, const char *end) {
    const size_t e = d.find(end, p);
    if (e == std::string::npos) throw XMLException("unterminated markup");
    return e + strlen(end);
  }
  static bool space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }
  static std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && space(s[a])) a++;
    while (b > a && space(s[b - 1])) b--;
    return s.substr(a, b - a);
  }
  static std::string decode(const std::string &v) {
    static const char *ent[][2] = {{"&amp;", "&"}, {"&lt;", "<"}, {"&gt;", ">"}, {"&quot;", "\""}, {"&apos;", "'"}};
    std::string out;
    for (size_t i = 0; i < v.size();) {
      bool hit = false;
      if (v[i] == '&')
        for (auto &e : ent)
          if (v.compare(i, strlen(e[0]), e[0]) == 0) {
            out += e[1];
            i += strlen(e[0]);
            hit = true;
            break;
          }
      if (!hit) out += v[i++];
    }
    return out;
  }
  size_t start_tag(const std::string &d, size_t p) {
    size_t q = p;
    while (q < d.size() && !space(d[q]) && d[q] != '>' && d[q] != '/') q++;
    const std::string name = d.substr(p, q - p);
    AttributeList atts;
    bool empty = false;
    for (;;) {
      while (q < d.size() && space(d[q])) q++;
      if (q >= d.size()) throw XMLException("unterminated start tag");
      if (d[q] == '>') {
        q++;
        break;
      }
      if (d[q] == '/') {
        empty = true;
        q = d.find('>', q);
        if (q == std::string::npos) throw XMLException("unterminated empty tag");
        q++;
        break;
      }
      size_t k = q;
      while (k < d.size() && !space(d[k]) && d[k] != '=') k++;
      const std::string key = d.substr(q, k - q);
      while (k < d.size() && space(d[k])) k++;
      if (k >= d.size() || d[k] != '=') throw XMLException("attribute without a value");
      k++;
      while (k < d.size() && space(d[k])) k++;
      if (k >= d.size() || (d[k] != '"' && d[k] != '\'')) throw XMLException("unquoted attribute value");
      const char quote = d[k];
      const size_t e = d.find(quote, k + 1);
      if (e == std::string::npos) throw XMLException("unterminated attribute value");
      atts.add(key, decode(d.substr(k + 1, e - k - 1)));
      q = e + 1;
    }
    XMLCh *x = oracle_shim::to_xml(name);
    if (handler_) {
      handler_->startElement(x, atts);
      if (empty) handler_->endElement(x);
    }
    return q;
  }

  HandlerBase *handler_ = nullptr;
};

#endif
