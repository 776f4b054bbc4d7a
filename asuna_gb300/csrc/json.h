// json.h — minimal JSON reader for Asuna scene files (objects, arrays,
// strings, numbers, booleans, null; UTF-8 passed through).
#pragma once
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace asuna {

struct Json {
  enum Type { Null, Bool, Number, String, Array, Object } type = Null;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;  // file order

  bool has(const std::string& k) const;
  const Json& operator[](const std::string& k) const;  // Null json if absent
  const Json& operator[](size_t i) const { return arr[i]; }
  size_t size() const { return type == Array ? arr.size() : (type == Object ? obj.size() : 0); }
  bool isNum() const { return type == Number; }
  bool isStr() const { return type == String; }
  bool isArr() const { return type == Array; }
  bool isObj() const { return type == Object; }
};

// Parses `text`; on error returns false and fills `err` with "line L: what".
bool parseJson(const std::string& text, Json& out, std::string& err);

}  // namespace asuna
