// Stand-in for the reference's VECTOR (src/rschol/linearalgebra/VECTOR.h:54-122):
// the members the adapter and the test driver use, same signatures.
#ifndef STANDIN_VECTOR_H
#define STANDIN_VECTOR_H
#include <cstring>
#include <vector>
#include <rschol/TYPES.h>

class VECTOR {
 public:
  VECTOR() : _size(0) {}
  VECTOR(int size) : _size(size), _store(size, 0.0) {}
  VECTOR(int size, const Real *data) : _size(size), _store(data, data + size) {}
  Real &operator()(int index) { return _store[index]; }
  Real operator()(int index) const { return _store[index]; }
  Real &operator[](int index) { return _store[index]; }
  int &size() { return _size; }
  int size() const { return _size; }
  void resizeAndWipe(int size) { _size = size; _store.assign(size, 0.0); }
  Real *data() { return _store.data(); }
  const Real *data() const { return _store.data(); }

 private:
  int _size;
  std::vector<Real> _store;
};
#endif
