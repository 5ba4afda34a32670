// Stand-in for the HDF5 C++ API, used only to compile the reference's own
// sources into the CPU oracle.  HDF5 checkpointing is not on the exact
// diagonalization path, so every operation throws: nothing here reads or
// writes a file.
#ifndef QCMG_ORACLE_H5CPP_STUB
#define QCMG_ORACLE_H5CPP_STUB

#include <string>
#include <stdexcept>
#include <cstdint>

typedef unsigned long long hsize_t;
typedef std::string H5std_string;

enum { H5F_ACC_RDONLY = 0, H5F_ACC_RDWR = 1, H5F_ACC_TRUNC = 2 };
enum { H5S_SCALAR = 0 };
static const size_t H5T_VARIABLE = (size_t)-1;

namespace H5 {

struct Exception {
  std::string msg{"HDF5 is not available in the oracle build"};
  std::string getDetailMsg() const { return msg; }
  const char* getCDetailMsg() const { return msg.c_str(); }
};

[[noreturn]] inline void unavailable() { throw Exception(); }

struct DataType {
  DataType() {}
  template <class... A> DataType(A&&...) {}
};
struct PredType : DataType {
  static const PredType NATIVE_DOUBLE, NATIVE_INT, C_S1, NATIVE_UINT64,
      NATIVE_INT64, NATIVE_UINT, NATIVE_CHAR;
};
inline const PredType PredType::NATIVE_DOUBLE{};
inline const PredType PredType::NATIVE_INT{};
inline const PredType PredType::C_S1{};
inline const PredType PredType::NATIVE_UINT64{};
inline const PredType PredType::NATIVE_INT64{};
inline const PredType PredType::NATIVE_UINT{};
inline const PredType PredType::NATIVE_CHAR{};
struct StrType : DataType {
  StrType() {}
  template <class... A> StrType(A&&...) {}
};

struct DataSpace {
  DataSpace() {}
  template <class... A> DataSpace(A&&...) {}
  template <class... A> int getSimpleExtentDims(A&&...) const { unavailable(); }
  int getSimpleExtentNdims() const { unavailable(); }
  void close() {}
};

struct Attribute {
  template <class... A> void read(A&&...) const { unavailable(); }
  template <class... A> void write(A&&...) const { unavailable(); }
  StrType getStrType() const { unavailable(); }
  DataSpace getSpace() const { unavailable(); }
  void close() {}
};

struct DataSet {
  template <class... A> void read(A&&...) const { unavailable(); }
  template <class... A> void write(A&&...) const { unavailable(); }
  DataSpace getSpace() const { unavailable(); }
  void close() {}
};

struct Group {
  Group() {}
  template <class... A> Group createGroup(A&&...) const { unavailable(); }
  template <class... A> Group openGroup(A&&...) const { unavailable(); }
  template <class... A> bool nameExists(A&&...) const { unavailable(); }
  template <class... A> bool attrExists(A&&...) const { unavailable(); }
  template <class... A> DataSet createDataSet(A&&...) const { unavailable(); }
  template <class... A> DataSet openDataSet(A&&...) const { unavailable(); }
  template <class... A> Attribute createAttribute(A&&...) const { unavailable(); }
  template <class... A> Attribute openAttribute(A&&...) const { unavailable(); }
  template <class... A> void unlink(A&&...) const { unavailable(); }
  void close() {}
};

struct H5File : Group {
  template <class... A> H5File(A&&...) { unavailable(); }
};

}  // namespace H5

#endif
