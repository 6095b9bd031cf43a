// Stand-in for tarch/la/Vector.h: a fixed-size vector with element access
// by [] and (), filled from one value or element by element.
#ifndef TARCH_LA_VECTOR_H_
#define TARCH_LA_VECTOR_H_
#include "peano/utils/Dimensions.h"

namespace tarch {
namespace la {

template <int Size, typename Scalar>
class Vector {
  Scalar _values[Size];

 public:
  Vector() {
    for (int i = 0; i < Size; i++) _values[i] = Scalar();
  }
  explicit Vector(const Scalar &value) {
    for (int i = 0; i < Size; i++) _values[i] = value;
  }
  Scalar &operator[](int i) { return _values[i]; }
  const Scalar &operator[](int i) const { return _values[i]; }
  Scalar &operator()(int i) { return _values[i]; }
  const Scalar &operator()(int i) const { return _values[i]; }
  int size() const { return Size; }
};

}  // namespace la
}  // namespace tarch
#endif
