// Minimal JSON reader for runmytrim input files.
//
// runmytrim reads its input with jsoncpp's default reader (apps/runmytrim.C:102-103),
// which accepts // and /* */ comments, trailing commas and text after the root
// value.  This reader accepts the same and offers the few queries the front-end
// needs: object members (the last one wins for duplicate keys, as in jsoncpp),
// arrays, numbers, strings and booleans.
#pragma once

#include <cstdlib>
#include <string>
#include <utility>
#include <vector>

namespace mtg_json
{

struct Value
{
  enum Kind
  {
    Null,
    Bool,
    Number,
    String,
    Array,
    Object
  };
  Kind kind = Null;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<Value> arr;
  std::vector<std::pair<std::string, Value>> obj;

  bool isObject() const { return kind == Object; }
  bool isArray() const { return kind == Array; }
  bool isNumeric() const { return kind == Number; }
  bool isString() const { return kind == String; }
  bool isBool() const { return kind == Bool; }
  // member `k` of an object, or a Null value
  const Value & operator[](const std::string & k) const
  {
    static const Value null_value;
    if (kind != Object)
      return null_value;
    for (size_t i = obj.size(); i-- > 0;)
      if (obj[i].first == k)
        return obj[i].second;
    return null_value;
  }
  const Value & operator[](size_t i) const
  {
    static const Value null_value;
    return kind == Array && i < arr.size() ? arr[i] : null_value;
  }
  size_t size() const { return kind == Array ? arr.size() : kind == Object ? obj.size() : 0; }
  double asDouble() const { return kind == Number ? num : kind == Bool ? (b ? 1.0 : 0.0) : 0.0; }
  long long asInt() const { return (long long)asDouble(); } // truncation, as jsoncpp
  bool asBool() const { return kind == Bool ? b : kind == Number ? num != 0.0 : false; }
  const std::string & asString() const { return str; }
};

class Parser
{
public:
  explicit Parser(const std::string & text) : s(text) {}

  bool parse(Value & out, std::string & err)
  {
    if (!value(out, 0))
    {
      err = msg + " at offset " + std::to_string(pos);
      return false;
    }
    return true; // text after the root value is ignored (jsoncpp failIfExtra = false)
  }

private:
  const std::string & s;
  size_t pos = 0;
  std::string msg;

  bool fail(const char * m)
  {
    msg = m;
    return false;
  }

  void skip()
  {
    while (pos < s.size())
    {
      const char c = s[pos];
      if (c == ' ' || c == '\t' || c == '\n' || c == '\r')
        ++pos;
      else if (c == '/' && pos + 1 < s.size() && s[pos + 1] == '/')
      {
        while (pos < s.size() && s[pos] != '\n')
          ++pos;
      }
      else if (c == '/' && pos + 1 < s.size() && s[pos + 1] == '*')
      {
        const size_t e = s.find("*/", pos + 2);
        pos = e == std::string::npos ? s.size() : e + 2;
      }
      else
        break;
    }
  }

  bool literal(const char * word)
  {
    const std::string w(word);
    if (s.compare(pos, w.size(), w) != 0)
      return false;
    pos += w.size();
    return true;
  }

  static void put_utf8(std::string & o, unsigned int cp)
  {
    if (cp < 0x80)
      o += char(cp);
    else if (cp < 0x800)
    {
      o += char(0xc0 | (cp >> 6));
      o += char(0x80 | (cp & 0x3f));
    }
    else if (cp < 0x10000)
    {
      o += char(0xe0 | (cp >> 12));
      o += char(0x80 | ((cp >> 6) & 0x3f));
      o += char(0x80 | (cp & 0x3f));
    }
    else
    {
      o += char(0xf0 | (cp >> 18));
      o += char(0x80 | ((cp >> 12) & 0x3f));
      o += char(0x80 | ((cp >> 6) & 0x3f));
      o += char(0x80 | (cp & 0x3f));
    }
  }

  bool hex4(unsigned int & v)
  {
    if (pos + 4 > s.size())
      return false;
    v = 0;
    for (int i = 0; i < 4; ++i)
    {
      const char c = s[pos++];
      v <<= 4;
      if (c >= '0' && c <= '9')
        v |= unsigned(c - '0');
      else if (c >= 'a' && c <= 'f')
        v |= unsigned(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F')
        v |= unsigned(c - 'A' + 10);
      else
        return false;
    }
    return true;
  }

  bool string(std::string & o)
  {
    ++pos; // opening quote
    while (pos < s.size())
    {
      const char c = s[pos++];
      if (c == '"')
        return true;
      if (c != '\\')
      {
        o += c;
        continue;
      }
      if (pos >= s.size())
        break;
      const char e = s[pos++];
      switch (e)
      {
        case '"': o += '"'; break;
        case '\\': o += '\\'; break;
        case '/': o += '/'; break;
        case 'b': o += '\b'; break;
        case 'f': o += '\f'; break;
        case 'n': o += '\n'; break;
        case 'r': o += '\r'; break;
        case 't': o += '\t'; break;
        case 'u':
        {
          unsigned int cp;
          if (!hex4(cp))
            return fail("bad \\u escape");
          if (cp >= 0xd800 && cp < 0xdc00 && pos + 1 < s.size() && s[pos] == '\\' && s[pos + 1] == 'u')
          {
            pos += 2;
            unsigned int lo;
            if (!hex4(lo) || lo < 0xdc00 || lo >= 0xe000)
              return fail("bad surrogate pair");
            cp = 0x10000 + ((cp - 0xd800) << 10) + (lo - 0xdc00);
          }
          put_utf8(o, cp);
          break;
        }
        default: return fail("bad escape");
      }
    }
    return fail("unterminated string");
  }

  bool number(Value & v)
  {
    const size_t start = pos;
    if (pos < s.size() && (s[pos] == '-' || s[pos] == '+'))
      ++pos;
    while (pos < s.size() && ((s[pos] >= '0' && s[pos] <= '9') || s[pos] == '.' || s[pos] == 'e' ||
                              s[pos] == 'E' || s[pos] == '-' || s[pos] == '+'))
      ++pos;
    const std::string tok = s.substr(start, pos - start);
    char * end = nullptr;
    v.num = std::strtod(tok.c_str(), &end);
    if (tok.empty() || !end || *end != '\0')
      return fail("bad number");
    v.kind = Value::Number;
    return true;
  }

  bool value(Value & v, int depth)
  {
    if (depth > 256)
      return fail("nesting too deep");
    skip();
    if (pos >= s.size())
      return fail("unexpected end of input");
    const char c = s[pos];
    if (c == '{')
    {
      ++pos;
      v.kind = Value::Object;
      skip();
      if (pos < s.size() && s[pos] == '}')
      {
        ++pos;
        return true;
      }
      while (true)
      {
        skip();
        if (pos < s.size() && s[pos] == '}') // trailing comma
        {
          ++pos;
          return true;
        }
        if (pos >= s.size() || s[pos] != '"')
          return fail("expected a member name");
        std::string key;
        if (!string(key))
          return false;
        skip();
        if (pos >= s.size() || s[pos] != ':')
          return fail("expected ':'");
        ++pos;
        Value m;
        if (!value(m, depth + 1))
          return false;
        v.obj.emplace_back(std::move(key), std::move(m));
        skip();
        if (pos < s.size() && s[pos] == ',')
        {
          ++pos;
          continue;
        }
        if (pos < s.size() && s[pos] == '}')
        {
          ++pos;
          return true;
        }
        return fail("expected ',' or '}'");
      }
    }
    if (c == '[')
    {
      ++pos;
      v.kind = Value::Array;
      skip();
      if (pos < s.size() && s[pos] == ']')
      {
        ++pos;
        return true;
      }
      while (true)
      {
        skip();
        if (pos < s.size() && s[pos] == ']') // trailing comma
        {
          ++pos;
          return true;
        }
        Value m;
        if (!value(m, depth + 1))
          return false;
        v.arr.push_back(std::move(m));
        skip();
        if (pos < s.size() && s[pos] == ',')
        {
          ++pos;
          continue;
        }
        if (pos < s.size() && s[pos] == ']')
        {
          ++pos;
          return true;
        }
        return fail("expected ',' or ']'");
      }
    }
    if (c == '"')
    {
      v.kind = Value::String;
      return string(v.str);
    }
    if (literal("true"))
    {
      v.kind = Value::Bool;
      v.b = true;
      return true;
    }
    if (literal("false"))
    {
      v.kind = Value::Bool;
      v.b = false;
      return true;
    }
    if (literal("null"))
    {
      v.kind = Value::Null;
      return true;
    }
    if (c == '-' || c == '+' || (c >= '0' && c <= '9') || c == '.')
      return number(v);
    return fail("unexpected character");
  }
};

inline bool
parse(const std::string & text, Value & out, std::string & err)
{
  Parser p(text);
  return p.parse(out, err);
}

} // namespace mtg_json
