// ORACLE — test infrastructure only: a stand-in for the header of the reference's sparse_matrix_math submodule
// (absent from the checkout), so that the reference's include/gpu_simulation_device.h can be compiled with
// -fsyntax-only against the C++ shim shown in INTEGRATION.md.  Declarations only, and only the members the
// reference's own call sites use: SMM::TripletMatrix iteration with getRow/getCol/getValue and the row, column
// and non-zero counts (cpp/gpu_sparse_matrix.cpp:7-50), addEntry/init (include/assembly.h:1022-1050).
#pragma once
#include <cstdint>

namespace SMM {

template <typename T>
class TripletMatrix {
public:
    class Triplet {
    public:
        int getRow() const;
        int getCol() const;
        T getValue() const;
    };
    class ConstIterator {
    public:
        const Triplet& operator*() const;
        const Triplet* operator->() const;
        ConstIterator& operator++();
        bool operator!=(const ConstIterator&) const;
    };
    void init(int rows, int cols, int nonZeros);
    void addEntry(int row, int col, T value);
    int getDenseRowCount() const;
    int getDenseColCount() const;
    int getNonZeroCount() const;
    ConstIterator begin() const;
    ConstIterator end() const;
};

}  // namespace SMM
