// TEST INFRASTRUCTURE ONLY: stand-in for h5rd, the HDF5 wrapper that ReaDDy's observable and IO code
// includes.  HDF5 is not installed in this image, so the types here have no file behind them: ReaDDy's
// sources compile against them, and any attempt to create, write or read a file throws.  The simulation
// path (neighbour list, forces, integration, reactions, observables kept in memory) never touches them.
#pragma once
#include <array>
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
[[noreturn]] inline void unavailable() { throw Exception("HDF5 files are not available in this build"); }

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
    const ParentFileRef &parentFile() const { return _parent; }
    ParentFileRef ref() const { return _parent; }

protected:
    ParentFileRef _parent;
};

class DataSetType : public Object {
public:
    DataSetType() = default;
    explicit DataSetType(ParentFileRef) {}
};
class NativeCompoundType : public DataSetType {};
class STDCompoundType : public DataSetType {
public:
    STDCompoundType() = default;
    explicit STDCompoundType(const NativeCompoundType &) {}
};
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
template <typename T, unsigned int N>
class NativeArrayDataSetType : public DataSetType {
public:
    explicit NativeArrayDataSetType(ParentFileRef = {}) {}
};
template <typename T, unsigned int N>
class STDArrayDataSetType : public DataSetType {
public:
    explicit STDArrayDataSetType(ParentFileRef = {}) {}
};

class NativeCompoundTypeBuilder {
public:
    NativeCompoundTypeBuilder(std::size_t, Object::ParentFileRef) {}
    template <typename T> NativeCompoundTypeBuilder &insert(const std::string &, std::size_t) { return *this; }
    NativeCompoundTypeBuilder &insertString(const std::string &, std::size_t) { return *this; }
    template <typename T, unsigned int N> NativeCompoundTypeBuilder &insertArray(const std::string &, std::size_t) { return *this; }
    template <typename T> NativeCompoundTypeBuilder &insertStdArray(const std::string &, std::size_t) { return *this; }
    NativeCompoundType build() { return {}; }
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
    template <typename T> void append(const dimensions &, std::vector<T> *) { unavailable(); }
    void flush() {}
};

class Group : public Object {
public:
    using FilterConfiguration = std::vector<Filter *>;
    Group createGroup(const std::string &) { unavailable(); }
    Group subgroup(const std::string &) { unavailable(); }
    Group getSubgroup(const std::string &) { unavailable(); }
    std::vector<std::string> containedDataSets() const { unavailable(); }
    template <typename T>
    std::unique_ptr<DataSet> createDataSet(const std::string &, const dimensions &, const dimensions &,
                                           const FilterConfiguration & = {}) { unavailable(); }
    std::unique_ptr<DataSet> createDataSet(const std::string &, const dimensions &, const dimensions &,
                                           const DataSetType &, const DataSetType &,
                                           const FilterConfiguration & = {}) { unavailable(); }
    template <typename T>
    std::unique_ptr<VLENDataSet> createVLENDataSet(const std::string &, const dimensions &, const dimensions &,
                                                   const FilterConfiguration & = {}) { unavailable(); }
    std::unique_ptr<VLENDataSet> createVLENDataSet(const std::string &, const dimensions &, const dimensions &,
                                                   const DataSetType &, const DataSetType &,
                                                   const FilterConfiguration & = {}) { unavailable(); }
    template <typename... A> void write(A &&...) { unavailable(); }
    template <typename T, typename... A> void read(const std::string &, T &, A...) { unavailable(); }
};

class File : public Group {
public:
    enum class Action { CREATE, OPEN };
    enum class Flag { READ_ONLY, READ_WRITE, OVERWRITE, FAIL_IF_EXISTS, CREATE_NON_EXISTING, DEFAULT };
    using Flags = std::vector<Flag>;
    static std::shared_ptr<File> open(const std::string &, const Flag & = Flag::READ_ONLY) { unavailable(); }
    static std::shared_ptr<File> create(const std::string &, const Flag & = Flag::OVERWRITE) { unavailable(); }
    void flush() {}
    void close() {}
};
}  // namespace h5rd
