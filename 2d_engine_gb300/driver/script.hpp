// script.hpp — reader for the reference's .sim script format (SCRIPT_READER.h/.cpp of
// ByungJoonLee/2D_Engine), with the same block/value access as its SCRIPT_BLOCK.
//
// Format: nested blocks `NAME { ... }` holding assignments `key = value`, where a value
// is true/false, a number, a vector `(a, b)` or a string "..."; `// ...` and `/* ... */`
// are comments; `#INCLUDE <file>` inlines another script (path relative to the
// including one); a `;` after a value is ignored.  FindBlock returns the first child of
// that name, or an empty block, so missing keys fall back to the caller's defaults just
// as SCRIPT_BLOCK's getters do (SCRIPT_READER.h:112-160).
#ifndef GB2D_SCRIPT_HPP
#define GB2D_SCRIPT_HPP

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace gb2d_script {

struct Block {
  std::string name;
  std::vector<std::pair<std::string, std::string>> values;  // in script order
  std::vector<std::unique_ptr<Block>> children;

  const Block& FindBlock(const std::string& n) const {
    for (const auto& c : children)
      if (c->name == n) return *c;
    return Empty();
  }
  bool Has(const std::string& key) const { return Find(key) != nullptr; }
  double GetFloat(const std::string& key, double dflt) const {
    const std::string* v = Find(key);
    return v ? std::strtod(v->c_str(), nullptr) : dflt;
  }
  int GetInteger(const std::string& key, int dflt) const {
    const std::string* v = Find(key);
    return v ? std::atoi(v->c_str()) : dflt;
  }
  bool GetBoolean(const std::string& key, bool dflt) const {
    const std::string* v = Find(key);
    return v ? *v == "true" : dflt;
  }
  std::string GetString(const std::string& key, const std::string& dflt) const {
    const std::string* v = Find(key);
    return v ? *v : dflt;
  }
  void GetVector2(const std::string& key, double& a, double& b) const {
    const std::string* v = Find(key);
    if (!v) return;
    std::string s = *v;
    for (char& ch : s)
      if (ch == '(' || ch == ')' || ch == ',') ch = ' ';
    std::istringstream in(s);
    in >> a >> b;
  }
  void GetInt2(const std::string& key, int& a, int& b) const {
    double x = a, y = b;
    GetVector2(key, x, y);
    a = (int)x;
    b = (int)y;
  }

  static const Block& Empty() {
    static const Block e;
    return e;
  }

 private:
  const std::string* Find(const std::string& key) const {
    for (const auto& kv : values)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
};

namespace detail {

inline std::string read_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open script " + path);
  std::ostringstream s;
  s << f.rdbuf();
  return s.str();
}

inline std::string dir_of(const std::string& path) {
  size_t k = path.find_last_of('/');
  return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

// Comments out, includes in.
inline std::string preprocess(const std::string& text, const std::string& dir, int depth) {
  if (depth > 16) throw std::runtime_error("#INCLUDE nested too deep");
  std::string out;
  for (size_t i = 0; i < text.size();) {
    if (text.compare(i, 2, "//") == 0) {
      while (i < text.size() && text[i] != '\n') ++i;
    } else if (text.compare(i, 2, "/*") == 0) {
      size_t e = text.find("*/", i + 2);
      i = e == std::string::npos ? text.size() : e + 2;
    } else if (text.compare(i, 8, "#INCLUDE") == 0) {
      size_t a = text.find('<', i), b = text.find('>', a == std::string::npos ? i : a);
      if (a == std::string::npos || b == std::string::npos) throw std::runtime_error("malformed #INCLUDE");
      std::string inc = text.substr(a + 1, b - a - 1);
      while (!inc.empty() && isspace((unsigned char)inc.back())) inc.pop_back();
      while (!inc.empty() && isspace((unsigned char)inc.front())) inc.erase(0, 1);
      std::string path = inc.size() && inc[0] == '/' ? inc : dir + inc;
      out += preprocess(read_file(path), dir_of(path), depth + 1);
      i = b + 1;
    } else {
      out += text[i++];
    }
  }
  return out;
}

struct Lexer {
  const std::string& s;
  size_t i = 0;
  explicit Lexer(const std::string& text) : s(text) {}
  void skip() {
    while (i < s.size() && (isspace((unsigned char)s[i]) || s[i] == ';')) ++i;
  }
  bool done() {
    skip();
    return i >= s.size();
  }
  char peek() {
    skip();
    return i < s.size() ? s[i] : '\0';
  }
  std::string word() {
    skip();
    size_t b = i;
    while (i < s.size() && (isalnum((unsigned char)s[i]) || s[i] == '_')) ++i;
    if (b == i) throw std::runtime_error("script: name expected near offset " + std::to_string(b));
    return s.substr(b, i - b);
  }
  std::string value() {
    skip();
    if (i >= s.size()) throw std::runtime_error("script: value expected");
    size_t b = i;
    if (s[i] == '(') {
      size_t e = s.find(')', i);
      if (e == std::string::npos) throw std::runtime_error("script: unterminated vector");
      i = e + 1;
      return s.substr(b, i - b);
    }
    if (s[i] == '"') {
      size_t e = s.find('"', i + 1);
      if (e == std::string::npos) throw std::runtime_error("script: unterminated string");
      i = e + 1;
      return s.substr(b + 1, e - b - 1);
    }
    while (i < s.size() && !isspace((unsigned char)s[i]) && s[i] != ';' && s[i] != '}' && s[i] != '{') ++i;
    return s.substr(b, i - b);
  }
  void expect(char c) {
    if (peek() != c) throw std::runtime_error(std::string("script: '") + c + "' expected near offset " + std::to_string(i));
    ++i;
  }
};

inline void parse_items(Lexer& lx, Block& into, bool top) {
  while (!lx.done()) {
    if (lx.peek() == '}') {
      if (top) throw std::runtime_error("script: unbalanced '}'");
      return;
    }
    std::string name = lx.word();
    char c = lx.peek();
    if (c == '=') {
      lx.expect('=');
      into.values.emplace_back(name, lx.value());
    } else if (c == '{') {
      lx.expect('{');
      std::unique_ptr<Block> child(new Block);
      child->name = name;
      parse_items(lx, *child, false);
      lx.expect('}');
      into.children.push_back(std::move(child));
    } else {
      throw std::runtime_error("script: '=' or '{' expected after " + name);
    }
  }
  if (!top) throw std::runtime_error("script: missing '}'");
}

}  // namespace detail

// The whole script as the children of one unnamed root block.
inline std::unique_ptr<Block> ReadScript(const std::string& path) {
  std::string text = detail::preprocess(detail::read_file(path), detail::dir_of(path), 0);
  std::unique_ptr<Block> root(new Block);
  detail::Lexer lx(text);
  detail::parse_items(lx, *root, true);
  return root;
}

}  // namespace gb2d_script

#endif  // GB2D_SCRIPT_HPP
