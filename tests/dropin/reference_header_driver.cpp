// Link check of the drop-in against the reference's own device-API header:
// this translation unit includes src/hmmLike.h unchanged (it declares the
// HMMLikeCUDA functions extern, hmmLike.h:23-38) and calls them in the order
// HMMLike's constructor and RunHMMOnSamples do (src/hmmLike.cpp:45-111); it
// links against include/hmmlike_cuda_shim.cpp and libglphase_gpu.so in place
// of src/hmmLike.cu.  Built only where the reference tree exists.
//
// Exit status: 0 when the whole sequence ran on a GPU; 3 when no device is
// visible and CheckDevice reported it as a std::runtime_error (the outcome on
// a machine without a GPU); 1 otherwise.
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "hmmLike.h"

int main() {
  const unsigned numSites = 256, numSamps = 2, numHaps = 8, numCycles = 4;
  std::vector<float> tran(3 * numSites, 0.f);
  for (unsigned m = 1; m < numSites; ++m) {
    tran[3 * m] = 0.98f;
    tran[3 * m + 1] = 0.0099f;
    tran[3 * m + 2] = 0.0002f;
  }
  float mut[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      mut[i][j] = i == j ? 0.97f : 0.01f;
  std::vector<std::pair<float, float> > codeBook(16, std::make_pair(1.f / 3, 1.f / 3));
  codeBook[0] = std::make_pair(1.f, 0.f);
  codeBook[1] = std::make_pair(0.f, 0.f);
  std::vector<uint32_t> packed(numSites / 8 * numSamps, 0x01230123u);
  std::vector<uint64_t> panel(numHaps * numSites / 64, 0x5555aaaa5555aaaaull);
  std::vector<unsigned> props(numSamps * numCycles), idx(4 * numSamps);
  for (unsigned i = 0; i < props.size(); ++i)
    props[i] = 4 + i % 4;
  for (unsigned i = 0; i < idx.size(); ++i)
    idx[i] = 4 + i % 4;
  try {
    HMMLikeCUDA::CheckDevice();
    HMMLikeCUDA::SetDevice(0);
    HMMLikeCUDA::CopyTranToDevice(tran);
    HMMLikeCUDA::CopyMutationMatToDevice(&mut);
    HMMLikeCUDA::CopyCodeBookToDevice(codeBook);
    HMMLikeCUDA::CopyPackedGLsToDevice(packed);
    HMMLikeCUDA::RunHMMOnDevice(panel, props, numSites, numSamps, numCycles, idx, 7ul);
    HMMLikeCUDA::Cleanup();
    for (unsigned v : idx)
      if (v >= numHaps)
        return 1;
    std::printf("ran on a device\n");
    return 0;
  } catch (const std::runtime_error &e) {
    std::printf("runtime_error: %s\n", e.what());
    return std::string(e.what()).find("no sm_103 device") != std::string::npos ? 3 : 1;
  }
}
