// Minimal stand-in for the flatbuffers runtime (test infrastructure for the reference pin).
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <vector>

namespace flatbuffers {
template <class T>
struct Offset {
  uint32_t o = 0;
};
template <class T>
struct Vector {
  uint32_t size() const { return 0; }
  T Get(uint32_t) const { return T(); }
  const T* begin() const { return nullptr; }
  const T* end() const { return nullptr; }
};
class FlatBufferBuilder {
 public:
  template <class T>
  void Finish(T) {}
  Offset<Vector<uint64_t>> CreateUninitializedVector(size_t n, size_t elem, uint8_t** p) {
    buf_.assign(n * elem + 1, 0);
    *p = buf_.data();
    return {};
  }
  template <class T>
  Offset<Vector<T>> CreateVectorOfStructs(const std::vector<T>&) { return {}; }
  uint8_t* GetBufferPointer() { return buf_.data(); }
  uint32_t GetSize() const { return (uint32_t)buf_.size(); }

 private:
  std::vector<uint8_t> buf_;
};
template <class T>
const T* GetRoot(const void* p) {
  return static_cast<const T*>(p);
}
}  // namespace flatbuffers
