// json.cpp — recursive-descent JSON reader (RFC 8259 subset: no surrogate
// pair decoding beyond the BMP, which scene files do not use).
#include "json.h"

#include <cstdlib>
#include <cstring>

namespace asuna {

static const Json kNullJson;

bool Json::has(const std::string& k) const {
  if (type != Object) return false;
  for (auto& kv : obj)
    if (kv.first == k) return true;
  return false;
}

const Json& Json::operator[](const std::string& k) const {
  if (type == Object)
    for (auto& kv : obj)
      if (kv.first == k) return kv.second;
  return kNullJson;
}

namespace {
struct Parser {
  const char* p;
  const char* end;
  const char* begin;
  std::string err;

  int line() const {
    int l = 1;
    for (const char* q = begin; q < p && q < end; ++q)
      if (*q == '\n') ++l;
    return l;
  }
  bool fail(const char* what) {
    if (err.empty()) err = "line " + std::to_string(line()) + ": " + what;
    return false;
  }
  void ws() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
  }
  bool lit(const char* s) {
    size_t n = std::strlen(s);
    if (size_t(end - p) >= n && std::strncmp(p, s, n) == 0) {
      p += n;
      return true;
    }
    return false;
  }
  static void utf8(std::string& o, unsigned cp) {
    if (cp < 0x80) {
      o += char(cp);
    } else if (cp < 0x800) {
      o += char(0xC0 | (cp >> 6));
      o += char(0x80 | (cp & 0x3F));
    } else {
      o += char(0xE0 | (cp >> 12));
      o += char(0x80 | ((cp >> 6) & 0x3F));
      o += char(0x80 | (cp & 0x3F));
    }
  }
  bool str(std::string& o) {
    if (p >= end || *p != '"') return fail("expected string");
    ++p;
    while (p < end && *p != '"') {
      if (*p == '\\') {
        ++p;
        if (p >= end) return fail("bad escape");
        char c = *p++;
        switch (c) {
          case '"': o += '"'; break;
          case '\\': o += '\\'; break;
          case '/': o += '/'; break;
          case 'b': o += '\b'; break;
          case 'f': o += '\f'; break;
          case 'n': o += '\n'; break;
          case 'r': o += '\r'; break;
          case 't': o += '\t'; break;
          case 'u': {
            if (end - p < 4) return fail("bad \\u escape");
            char hex[5] = {p[0], p[1], p[2], p[3], 0};
            p += 4;
            utf8(o, unsigned(std::strtoul(hex, nullptr, 16)));
            break;
          }
          default: return fail("bad escape");
        }
      } else {
        o += *p++;
      }
    }
    if (p >= end) return fail("unterminated string");
    ++p;
    return true;
  }
  bool value(Json& v, int depth) {
    if (depth > 256) return fail("nesting too deep");
    ws();
    if (p >= end) return fail("unexpected end of input");
    char c = *p;
    if (c == '{') {
      ++p;
      v.type = Json::Object;
      ws();
      if (p < end && *p == '}') {
        ++p;
        return true;
      }
      for (;;) {
        ws();
        std::string k;
        if (!str(k)) return false;
        ws();
        if (p >= end || *p != ':') return fail("expected ':'");
        ++p;
        Json child;
        if (!value(child, depth + 1)) return false;
        v.obj.emplace_back(std::move(k), std::move(child));
        ws();
        if (p < end && *p == ',') {
          ++p;
          continue;
        }
        if (p < end && *p == '}') {
          ++p;
          return true;
        }
        return fail("expected ',' or '}'");
      }
    }
    if (c == '[') {
      ++p;
      v.type = Json::Array;
      ws();
      if (p < end && *p == ']') {
        ++p;
        return true;
      }
      for (;;) {
        Json child;
        if (!value(child, depth + 1)) return false;
        v.arr.push_back(std::move(child));
        ws();
        if (p < end && *p == ',') {
          ++p;
          continue;
        }
        if (p < end && *p == ']') {
          ++p;
          return true;
        }
        return fail("expected ',' or ']'");
      }
    }
    if (c == '"') {
      v.type = Json::String;
      return str(v.str);
    }
    if (lit("true")) {
      v.type = Json::Bool;
      v.b = true;
      return true;
    }
    if (lit("false")) {
      v.type = Json::Bool;
      v.b = false;
      return true;
    }
    if (lit("null")) {
      v.type = Json::Null;
      return true;
    }
    if (c == '-' || (c >= '0' && c <= '9')) {
      char* e = nullptr;
      std::string tmp(p, size_t(std::min<ptrdiff_t>(end - p, 64)));
      double d = std::strtod(tmp.c_str(), &e);
      if (e == tmp.c_str()) return fail("bad number");
      p += (e - tmp.c_str());
      v.type = Json::Number;
      v.num = d;
      return true;
    }
    return fail("unexpected character");
  }
};
}  // namespace

bool parseJson(const std::string& text, Json& out, std::string& err) {
  Parser ps{text.data(), text.data() + text.size(), text.data(), {}};
  out = Json();
  if (!ps.value(out, 0)) {
    err = ps.err;
    return false;
  }
  ps.ws();
  if (ps.p != ps.end) {
    ps.fail("trailing characters");
    err = ps.err;
    return false;
  }
  return true;
}

}  // namespace asuna
