// From-scratch stand-in for asl/Xml.h (see defs.h): a small XML element tree.
// Restated semantics: Xml::read parses elements and attributes (prolog,
// comments, DOCTYPE and CDATA skipped; text ignored; &quot; &apos; &lt; &gt;
// &amp; decoded in attribute values); e["a"] is attribute a ("" if absent);
// e("t") is the first child element with tag t; findOne(p) is the first
// element, in document order starting with this one, for which p holds.
#ifndef ASL_SHIM_XML_H
#define ASL_SHIM_XML_H
#include "defs.h"
#include "String.h"
#include <memory>
#include <string>
#include <vector>
namespace asl {
class Xml {
  struct Node {
    std::string tag;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<std::shared_ptr<Node>> kids;
  };
  std::shared_ptr<Node> n_;
  explicit Xml(std::shared_ptr<Node> n) : n_(n) {}

  static std::string decode(const std::string& s) {
    std::string r;
    for (size_t i = 0; i < s.size(); i++) {
      if (s[i] == '&') {
        size_t e = s.find(';', i);
        if (e != std::string::npos) {
          std::string ent = s.substr(i + 1, e - i - 1);
          const char* rep = ent == "quot" ? "\"" : ent == "apos" ? "'" : ent == "lt" ? "<" : ent == "gt" ? ">"
                            : ent == "amp" ? "&" : nullptr;
          if (rep) { r += rep; i = e; continue; }
        }
      }
      r += s[i];
    }
    return r;
  }
  struct Parser {
    const std::string& s;
    size_t i = 0;
    explicit Parser(const std::string& t) : s(t) {}
    bool starts(const char* p) const { return s.compare(i, strlen(p), p) == 0; }
    void skip_ws() { while (i < s.size() && isspace((unsigned char)s[i])) i++; }
    void skip_misc() {  // text, comments, prolog, DOCTYPE, CDATA between elements
      for (;;) {
        while (i < s.size() && s[i] != '<') i++;
        if (i >= s.size()) return;
        if (starts("<!--")) { size_t e = s.find("-->", i); i = e == std::string::npos ? s.size() : e + 3; }
        else if (starts("<![CDATA[")) { size_t e = s.find("]]>", i); i = e == std::string::npos ? s.size() : e + 3; }
        else if (starts("<?")) { size_t e = s.find("?>", i); i = e == std::string::npos ? s.size() : e + 2; }
        else if (starts("<!")) {
          int depth = 0;
          for (; i < s.size(); i++) {
            if (s[i] == '[') depth++;
            else if (s[i] == ']') depth--;
            else if (s[i] == '>' && depth <= 0) { i++; break; }
          }
        } else return;
      }
    }
    std::shared_ptr<Node> element() {  // at '<' of a start tag
      auto n = std::make_shared<Node>();
      i++;
      size_t b = i;
      while (i < s.size() && !isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/') i++;
      n->tag = s.substr(b, i - b);
      for (;;) {
        skip_ws();
        if (i >= s.size()) return n;
        if (s[i] == '/') { i = s.find('>', i); i = i == std::string::npos ? s.size() : i + 1; return n; }
        if (s[i] == '>') { i++; break; }
        size_t a = i;
        while (i < s.size() && s[i] != '=' && !isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/') i++;
        std::string name = s.substr(a, i - a);
        skip_ws();
        std::string val;
        if (i < s.size() && s[i] == '=') {
          i++;
          skip_ws();
          char q = i < s.size() ? s[i] : 0;
          if (q == '"' || q == '\'') {
            size_t e = s.find(q, i + 1);
            if (e == std::string::npos) e = s.size();
            val = decode(s.substr(i + 1, e - i - 1));
            i = e + 1;
          }
        }
        if (!name.empty()) n->attrs.push_back({name, val});
      }
      for (;;) {  // children until the end tag
        skip_misc();
        if (i >= s.size()) return n;
        if (starts("</")) { i = s.find('>', i); i = i == std::string::npos ? s.size() : i + 1; return n; }
        n->kids.push_back(element());
      }
    }
  };
  template <class F> static std::shared_ptr<Node> find(const std::shared_ptr<Node>& n, F& pred) {
    if (pred(Xml(n))) return n;
    for (auto& k : n->kids) {
      auto r = find(k, pred);
      if (r) return r;
    }
    return nullptr;
  }

 public:
  Xml() {}
  static Xml read(const String& filename) {
    FILE* f = fopen(*filename, "rb");
    if (!f) return Xml();
    std::string t;
    char buf[65536];
    size_t k;
    while ((k = fread(buf, 1, sizeof buf, f)) > 0) t.append(buf, k);
    fclose(f);
    Parser p(t);
    p.skip_misc();
    if (p.i >= t.size()) return Xml();
    return Xml(p.element());
  }
  explicit operator bool() const { return (bool)n_; }
  bool operator!() const { return !n_; }
  String tag() const { return n_ ? String(n_->tag) : String(); }
  bool has(const char* a) const {
    if (n_) for (auto& kv : n_->attrs) if (kv.first == a) return true;
    return false;
  }
  String operator[](const char* a) const {
    if (n_) for (auto& kv : n_->attrs) if (kv.first == a) return String(kv.second);
    return String();
  }
  Xml operator()(const char* t) const {
    if (n_) for (auto& k : n_->kids) if (k->tag == t) return Xml(k);
    return Xml();
  }
  Array<Xml> children() const {
    Array<Xml> out;
    if (n_) for (auto& k : n_->kids) out << Xml(k);
    return out;
  }
  template <class F> Xml findOne(F pred) const { return n_ ? Xml(find(n_, pred)) : Xml(); }
};
}  // namespace asl
#endif
