// TEST INFRASTRUCTURE ONLY: a small stand-in for the nlohmann JSON library, which ReaDDy's kernel
// configuration, timer and IO sources use and which is not installed in this image.  It is written for
// this repository and offers only what those sources call: a JSON value (null, bool, number, string,
// array, object) built from numbers, strings, std::array/std::vector, initializer lists (an object when
// every element is a [string, value] pair, an array otherwise) and types with an ADL to_json; operator[],
// at, find/end, get<T> (numbers, strings, bool, and types with an ADL from_json), implicit conversion,
// parse and dump.
#pragma once
#include <array>
#include <cstdint>
#include <cstdio>
#include <initializer_list>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace nlohmann {

class json;

namespace detail {
template <typename T, typename = void>
struct has_to_json : std::false_type {};
template <typename T>
struct has_to_json<T, std::void_t<decltype(to_json(std::declval<json &>(), std::declval<const T &>()))>> : std::true_type {};
template <typename T>
struct is_sequence : std::false_type {};
template <typename T, std::size_t N>
struct is_sequence<std::array<T, N>> : std::true_type {};
template <typename T, typename A>
struct is_sequence<std::vector<T, A>> : std::true_type {};
}  // namespace detail

class json {
public:
    enum class kind { null, boolean, number, string, array, object };
    using object_t = std::vector<std::pair<std::string, json>>;
    using const_iterator = const std::pair<std::string, json> *;

    json() = default;
    json(std::nullptr_t) {}
    json(bool b) : _k(kind::boolean), _b(b) {}
    template <typename T, std::enable_if_t<std::is_arithmetic_v<T> && !std::is_same_v<T, bool>, int> = 0>
    json(T v) : _k(kind::number), _n((double)v) {}
    json(const char *s) : _k(kind::string), _s(s) {}
    json(std::string s) : _k(kind::string), _s(std::move(s)) {}
    template <typename T, std::enable_if_t<detail::is_sequence<T>::value, int> = 0>
    json(const T &seq) : _k(kind::array) {
        for (const auto &v : seq) _a.emplace_back(v);
    }
    template <typename T, std::enable_if_t<!std::is_arithmetic_v<T> && !detail::is_sequence<T>::value &&
                                               !std::is_same_v<std::decay_t<T>, json> && detail::has_to_json<T>::value,
                                           int> = 0>
    json(const T &v) {
        to_json(*this, v);
    }
    json(std::initializer_list<json> items) {
        bool pairs = items.size() > 0;
        for (const auto &e : items) pairs &= e._k == kind::array && e._a.size() == 2 && e._a[0]._k == kind::string;
        if (pairs) {
            _k = kind::object;
            for (const auto &e : items) (*this)[e._a[0]._s] = e._a[1];
        } else {
            _k = kind::array;
            _a.assign(items.begin(), items.end());
        }
    }

    json &operator[](const std::string &key) {
        if (_k == kind::null) _k = kind::object;
        if (_k != kind::object) throw std::domain_error("json: operator[] on a value that is not an object");
        for (auto &e : _o) if (e.first == key) return e.second;
        _o.emplace_back(key, json());
        return _o.back().second;
    }
    const json &at(const std::string &key) const {
        for (const auto &e : _o) if (e.first == key) return e.second;
        throw std::out_of_range("json: key '" + key + "' not found");
    }
    const_iterator find(const std::string &key) const {
        for (const auto &e : _o) if (e.first == key) return &e;
        return end();
    }
    const_iterator end() const { return _o.data() + _o.size(); }

    template <typename T>
    T get() const {
        if constexpr (std::is_same_v<T, bool>) {
            return _b;
        } else if constexpr (std::is_arithmetic_v<T>) {
            return (T)_n;
        } else if constexpr (std::is_same_v<T, std::string>) {
            return _s;
        } else {
            T v{};
            from_json(*this, v);
            return v;
        }
    }
    template <typename T, std::enable_if_t<!std::is_same_v<T, json> && !std::is_reference_v<T>, int> = 0>
    operator T() const {
        return get<T>();
    }

    static json parse(const std::string &text) {
        std::size_t at = 0;
        json v = parse_value(text, at);
        skip(text, at);
        if (at != text.size()) throw std::invalid_argument("json: trailing characters");
        return v;
    }

    std::string dump() const {
        switch (_k) {
            case kind::null: return "null";
            case kind::boolean: return _b ? "true" : "false";
            case kind::number: {
                char buf[64];
                std::snprintf(buf, sizeof buf, "%.17g", _n);
                return buf;
            }
            case kind::string: return "\"" + _s + "\"";
            case kind::array: {
                std::string r = "[";
                for (std::size_t i = 0; i < _a.size(); ++i) r += (i ? "," : "") + _a[i].dump();
                return r + "]";
            }
            case kind::object: {
                std::string r = "{";
                for (std::size_t i = 0; i < _o.size(); ++i) r += (i ? ",\"" : "\"") + _o[i].first + "\":" + _o[i].second.dump();
                return r + "}";
            }
        }
        return "null";
    }

private:
    static void skip(const std::string &t, std::size_t &i) {
        while (i < t.size() && (t[i] == ' ' || t[i] == '\n' || t[i] == '\t' || t[i] == '\r')) ++i;
    }
    static json parse_value(const std::string &t, std::size_t &i) {
        skip(t, i);
        if (i >= t.size()) throw std::invalid_argument("json: unexpected end");
        const char c = t[i];
        if (c == '{') {
            json o;
            o._k = kind::object;
            ++i;
            skip(t, i);
            if (i < t.size() && t[i] == '}') { ++i; return o; }
            for (;;) {
                skip(t, i);
                const std::string key = parse_value(t, i)._s;
                skip(t, i);
                if (i >= t.size() || t[i++] != ':') throw std::invalid_argument("json: expected ':'");
                o[key] = parse_value(t, i);
                skip(t, i);
                if (i < t.size() && t[i] == ',') { ++i; continue; }
                if (i < t.size() && t[i] == '}') { ++i; return o; }
                throw std::invalid_argument("json: expected ',' or '}'");
            }
        }
        if (c == '[') {
            json a;
            a._k = kind::array;
            ++i;
            skip(t, i);
            if (i < t.size() && t[i] == ']') { ++i; return a; }
            for (;;) {
                a._a.push_back(parse_value(t, i));
                skip(t, i);
                if (i < t.size() && t[i] == ',') { ++i; continue; }
                if (i < t.size() && t[i] == ']') { ++i; return a; }
                throw std::invalid_argument("json: expected ',' or ']'");
            }
        }
        if (c == '"') {
            std::string s;
            for (++i; i < t.size() && t[i] != '"'; ++i) {
                if (t[i] == '\\' && i + 1 < t.size()) ++i;
                s += t[i];
            }
            ++i;
            return json(std::move(s));
        }
        if (t.compare(i, 4, "true") == 0) { i += 4; return json(true); }
        if (t.compare(i, 5, "false") == 0) { i += 5; return json(false); }
        if (t.compare(i, 4, "null") == 0) { i += 4; return json(); }
        std::size_t used = 0;
        const double v = std::stod(t.substr(i), &used);
        i += used;
        return json(v);
    }

    kind _k = kind::null;
    bool _b = false;
    double _n = 0;
    std::string _s;
    std::vector<json> _a;
    object_t _o;
};

}  // namespace nlohmann
