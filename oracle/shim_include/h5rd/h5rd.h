// TEST INFRASTRUCTURE ONLY: stand-in for h5rd, the HDF5 wrapper that ReaDDy's observable and IO headers
// include.  HDF5 is not installed in this image, so the types are declared without a file behind them:
// ReaDDy's headers compile, and any attempt to open or write a file throws.  Nothing on the simulation
// path (neighbour list, forces, integration, reactions) touches these types.
#pragma once
#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace h5rd {
using handle_id = std::int64_t;
using dimension = unsigned long long;
using dimensions = std::vector<dimension>;
constexpr dimension UNLIMITED_DIMS = ~0ull;

struct Exception : std::runtime_error {
    using std::runtime_error::runtime_error;
};
[[noreturn]] inline void unavailable() { throw Exception("HDF5 output is not available in this build"); }

class File;
class PropertyList {};
class Filter {
public:
    virtual ~Filter() = default;
    virtual bool available() const = 0;
    virtual void activate(PropertyList &plist) = 0;
    virtual void registerFilter() = 0;
};

class Object {
public:
    using ParentFileRef = std::shared_ptr<File>;
    virtual ~Object() = default;
};

class DataSetType : public Object {};
class NativeCompoundType : public DataSetType {};
class STDCompoundType : public DataSetType {};
template <typename T>
class NativeDataSetType : public DataSetType {
public:
    explicit NativeDataSetType(ParentFileRef = {}) {}
};
template <typename T>
class STDDataSetType : public DataSetType {
public:
    explicit STDDataSetType(ParentFileRef = {}) {}
};

class DataSet : public Object {
public:
    template <typename T> void append(std::vector<T> &) { unavailable(); }
    template <typename T> void append(const dimensions &, const T *) { unavailable(); }
    void flush() {}
};
class VLENDataSet : public Object {
public:
    template <typename T> void append(std::vector<std::vector<T>> &) { unavailable(); }
    void flush() {}
};

class Group : public Object {
public:
    Group subgroup(const std::string &) { unavailable(); }
    Group createGroup(const std::string &) { unavailable(); }
};

class File : public Group {
public:
    enum class Flag { READ_ONLY, READ_WRITE, OVERWRITE, FAIL_IF_EXISTS, CREATE_NON_EXISTING, DEFAULT };
    static std::shared_ptr<File> open(const std::string &, const Flag & = Flag::READ_ONLY) { unavailable(); }
    static std::shared_ptr<File> create(const std::string &, const Flag & = Flag::OVERWRITE) { unavailable(); }
    void flush() {}
    void close() {}
};
}  // namespace h5rd
