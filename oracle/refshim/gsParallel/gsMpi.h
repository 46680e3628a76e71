// Test-only stand-in for gismo's serial communicator (the build without MPI): one process.
#pragma once

namespace gismo {

class gsSerialComm {
public:
    int rank() const { return 0; }
    int size() const { return 1; }
    void barrier() const {}
};

}  // namespace gismo
