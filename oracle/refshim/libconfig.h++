/*
 * Minimal stand-in for libconfig++ -- TEST INFRASTRUCTURE ONLY.
 *
 * It lets the reference's SimParams (src/SimParams.cpp:45-468) read .cfg files unchanged in
 * the reference build under oracle/_ref.  It parses the libconfig grammar the reference's
 * files use -- groups { }, lists ( ), arrays [ ], `name = value;` or `name : value;`,
 * integers (decimal, hex), floats, booleans, strings (adjacent literals concatenate),
 * comments `#`, `//`, `/ * * /` -- and types values the way libconfig does with automatic
 * conversion off (its default): an integer setting does not read as a double and a float
 * does not read as an integer.  Only the calls the reference makes are provided.
 */
#ifndef IMPEC_REFSHIM_LIBCONFIG_HPP
#define IMPEC_REFSHIM_LIBCONFIG_HPP

#include <cctype>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace libconfig {

class ConfigException : public std::exception {
public:
    const char* what() const noexcept override { return "ConfigException"; }
};
class FileIOException : public ConfigException {
public:
    const char* what() const noexcept override { return "FileIOException"; }
};
class ParseException : public ConfigException {
public:
    ParseException(const std::string& file, int line, const std::string& err) : file_(file), line_(line), err_(err) {}
    const char* getFile() const { return file_.c_str(); }
    int getLine() const { return line_; }
    const char* getError() const { return err_.c_str(); }
    const char* what() const noexcept override { return "ParseException"; }

private:
    std::string file_;
    int line_;
    std::string err_;
};
class SettingException : public ConfigException {
public:
    explicit SettingException(const std::string& path) : path_(path) {}
    const char* getPath() const { return path_.c_str(); }

private:
    std::string path_;
};
class SettingNotFoundException : public SettingException {
public:
    using SettingException::SettingException;
    const char* what() const noexcept override { return "SettingNotFoundException"; }
};
class SettingTypeException : public SettingException {
public:
    using SettingException::SettingException;
    const char* what() const noexcept override { return "SettingTypeException"; }
};

class Setting {
public:
    enum Type { TypeNone, TypeGroup, TypeInt, TypeInt64, TypeFloat, TypeString, TypeBoolean, TypeArray, TypeList };

    Type getType() const { return type_; }
    const char* getName() const { return name_.c_str(); }
    std::string getPath() const { return path_; }
    int getLength() const { return (int)children_.size(); }
    bool isGroup() const { return type_ == TypeGroup; }
    bool isList() const { return type_ == TypeList; }
    bool isArray() const { return type_ == TypeArray; }
    bool isNumber() const { return type_ == TypeInt || type_ == TypeInt64 || type_ == TypeFloat; }
    bool exists(const char* name) const { return find(name) != nullptr; }
    bool exists(const std::string& name) const { return exists(name.c_str()); }

    const Setting& operator[](const char* name) const {
        const Setting* s = find(name);
        if (!s) throw SettingNotFoundException(path_ + "." + name);
        return *s;
    }
    const Setting& operator[](const std::string& name) const { return (*this)[name.c_str()]; }
    const Setting& operator[](int i) const {
        if (i < 0 || i >= (int)children_.size()) throw SettingNotFoundException(path_ + "[" + std::to_string(i) + "]");
        return *children_[i];
    }

    operator int() const {
        want(TypeInt);
        return (int)ival_;
    }
    operator long() const {
        want(TypeInt);
        return (long)ival_;
    }
    operator long long() const {
        want(TypeInt);
        return ival_;
    }
    operator unsigned int() const {
        want(TypeInt);
        return (unsigned int)ival_;
    }
    operator double() const {
        want(TypeFloat);
        return fval_;
    }
    operator float() const {
        want(TypeFloat);
        return (float)fval_;
    }
    operator bool() const {
        want(TypeBoolean);
        return bval_;
    }
    operator std::string() const {
        want(TypeString);
        return sval_;
    }
    operator const char*() const {
        want(TypeString);
        return sval_.c_str();
    }

    template <typename T>
    bool lookupValue(const char* name, T& value) const {
        try {
            value = convert<T>((*this)[name]);
            return true;
        } catch (const ConfigException&) {
            return false;
        }
    }
    template <typename T>
    bool lookupValue(const std::string& name, T& value) const {
        return lookupValue(name.c_str(), value);
    }

    // --- construction (used by the parser) ---
    Type type_ = TypeNone;
    std::string name_, path_;
    long long ival_ = 0;
    double fval_ = 0;
    bool bval_ = false;
    std::string sval_;
    std::vector<std::unique_ptr<Setting>> children_;

private:
    template <typename T>
    static T convert(const Setting& s) {
        return static_cast<T>(s);
    }
    void want(Type t) const {
        Type have = type_ == TypeInt64 ? TypeInt : type_;
        if (have != t) throw SettingTypeException(path_);
    }
    const Setting* find(const char* name) const {
        if (type_ != TypeGroup) return nullptr;
        for (const auto& c : children_)
            if (c->name_ == name) return c.get();
        return nullptr;
    }
};

template <>
inline std::string Setting::convert<std::string>(const Setting& s) {
    return s.operator std::string();
}

class Config {
public:
    Config() { root_.type_ = Setting::TypeGroup; }
    void setAutoConvert(bool) {}
    const Setting& getRoot() const { return root_; }
    void readFile(const char* path) {
        std::ifstream f(path);
        if (!f) throw FileIOException();
        std::stringstream ss;
        ss << f.rdbuf();
        Parser p(ss.str(), path);
        root_.children_.clear();
        p.group_body(root_, '\0');
    }
    template <typename T>
    bool lookupValue(const char* path, T& value) const {
        const Setting* s = &root_;
        std::string part;
        std::stringstream ps(path);
        while (std::getline(ps, part, '.')) {
            if (!s->exists(part.c_str())) return false;
            s = &(*s)[part.c_str()];
        }
        try {
            value = static_cast<T>(*s);
            return true;
        } catch (const ConfigException&) {
            return false;
        }
    }
    bool exists(const char* path) const {
        const Setting* s = &root_;
        std::string part;
        std::stringstream ps(path);
        while (std::getline(ps, part, '.')) {
            if (!s->exists(part.c_str())) return false;
            s = &(*s)[part.c_str()];
        }
        return true;
    }

private:
    Setting root_;

    struct Parser {
        std::string text;
        std::string file;
        size_t pos = 0;
        int line = 1;
        Parser(const std::string& t, const std::string& f) : text(t), file(f) {}

        [[noreturn]] void fail(const std::string& msg) { throw ParseException(file, line, msg); }
        void skip() {
            for (;;) {
                while (pos < text.size() && std::isspace((unsigned char)text[pos])) {
                    if (text[pos] == '\n') ++line;
                    ++pos;
                }
                if (pos < text.size() && text[pos] == '#') {
                    while (pos < text.size() && text[pos] != '\n') ++pos;
                } else if (text.compare(pos, 2, "//") == 0) {
                    while (pos < text.size() && text[pos] != '\n') ++pos;
                } else if (text.compare(pos, 2, "/*") == 0) {
                    size_t e = text.find("*/", pos + 2);
                    if (e == std::string::npos) fail("unterminated comment");
                    for (size_t k = pos; k < e; ++k)
                        if (text[k] == '\n') ++line;
                    pos = e + 2;
                } else {
                    return;
                }
            }
        }
        char peek() {
            skip();
            return pos < text.size() ? text[pos] : '\0';
        }
        std::string name() {
            skip();
            size_t s = pos;
            while (pos < text.size() && (std::isalnum((unsigned char)text[pos]) || text[pos] == '_' || text[pos] == '-' ||
                                         text[pos] == '*'))
                ++pos;
            if (s == pos) fail("expected a setting name");
            return text.substr(s, pos - s);
        }
        void group_body(Setting& g, char close) {
            for (;;) {
                char c = peek();
                if (c == close) {
                    if (close) ++pos;
                    return;
                }
                if (c == '\0') fail("unexpected end of file");
                auto child = std::unique_ptr<Setting>(new Setting());
                child->name_ = name();
                child->path_ = g.path_.empty() ? child->name_ : g.path_ + "." + child->name_;
                c = peek();
                if (c != '=' && c != ':') fail("expected = or :");
                ++pos;
                value(*child);
                c = peek();
                if (c == ';' || c == ',') ++pos;
                g.children_.push_back(std::move(child));
            }
        }
        void value(Setting& s) {
            char c = peek();
            if (c == '{') {
                ++pos;
                s.type_ = Setting::TypeGroup;
                group_body(s, '}');
            } else if (c == '(' || c == '[') {
                ++pos;
                const char close = c == '(' ? ')' : ']';
                s.type_ = c == '(' ? Setting::TypeList : Setting::TypeArray;
                for (int k = 0;; ++k) {
                    if (peek() == close) {
                        ++pos;
                        return;
                    }
                    auto e = std::unique_ptr<Setting>(new Setting());
                    e->path_ = s.path_ + "[" + std::to_string(k) + "]";
                    value(*e);
                    s.children_.push_back(std::move(e));
                    char d = peek();
                    if (d == ',') ++pos;
                    else if (d != close) fail("expected , or closing bracket");
                }
            } else if (c == '"') {
                s.type_ = Setting::TypeString;
                while (peek() == '"') {
                    ++pos;
                    while (pos < text.size() && text[pos] != '"') {
                        char ch = text[pos++];
                        if (ch == '\\' && pos < text.size()) {
                            char e = text[pos++];
                            ch = e == 'n' ? '\n' : e == 't' ? '\t' : e == 'r' ? '\r' : e == 'f' ? '\f' : e;
                        }
                        s.sval_.push_back(ch);
                    }
                    if (pos >= text.size()) fail("unterminated string");
                    ++pos;
                }
            } else {
                skip();
                size_t st = pos;
                while (pos < text.size() && (std::isalnum((unsigned char)text[pos]) || text[pos] == '.' ||
                                             text[pos] == '+' || text[pos] == '-'))
                    ++pos;
                std::string tok = text.substr(st, pos - st);
                if (tok.empty()) fail("expected a value");
                std::string low;
                for (char ch : tok) low.push_back((char)std::tolower((unsigned char)ch));
                if (low == "true" || low == "false") {
                    s.type_ = Setting::TypeBoolean;
                    s.bval_ = low == "true";
                    return;
                }
                bool hex = low.size() > 2 && (low.compare(0, 2, "0x") == 0 || low.compare(0, 3, "-0x") == 0);
                bool is_float = !hex && (low.find_first_of(".e") != std::string::npos);
                while (!low.empty() && low.back() == 'l') low.pop_back();  // 64-bit suffix
                char* end = nullptr;
                if (is_float) {
                    s.type_ = Setting::TypeFloat;
                    s.fval_ = std::strtod(low.c_str(), &end);
                } else {
                    s.type_ = Setting::TypeInt;
                    s.ival_ = std::strtoll(low.c_str(), &end, hex ? 16 : 10);
                }
                if (!end || *end != '\0') fail("bad number '" + tok + "'");
            }
        }
    };
};

}  // namespace libconfig

#endif
