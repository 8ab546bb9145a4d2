// The reference's example program (Example/examPointCloud/examPointCloud.cpp:54-132)
// written against this library's ophPointCloud class, unchanged in its call
// sequence: readConfig -> loadPointCloud -> SetMode(MODE_GPU) ->
// generateHologram(PC_DIFF_RS) -> saveAsOhc -> encoding(ENCODE_PHASE) ->
// normalize -> save -> release. Built and run by tests/test_cpp_dropin_gpu.py.
//
//   exam_pointcloud <config.xml> <cloud.ply> <output directory>
#include "ophPointCloud.h"

#include <iostream>
#include <string>

int main(int argc, char** argv) {
    if (argc != 4) {
        std::cerr << "usage: exam_pointcloud <config.xml> <cloud.ply> <output directory>" << std::endl;
        return 2;
    }
    ophPointCloud* Hologram = new ophPointCloud();
    if (!Hologram->readConfig(argv[1])) {
        std::cerr << "Fail to load Config file : " << argv[1] << std::endl;
        return 1;
    }
    if (Hologram->loadPointCloud(argv[2]) < 0) {
        std::cerr << "Fail to load Point Cloud file : " << argv[2] << std::endl;
        return 1;
    }
    Hologram->SetMode(MODE_GPU);
    if (Hologram->generateHologram(ophPointCloud::PC_DIFF_FLAG::PC_DIFF_RS) <= 0.0) {
        std::cerr << "generateHologram failed: " << Hologram->lastError() << std::endl;
        return 1;
    }
    const std::string res = std::string(argv[3]) + "/";
    if (!Hologram->saveAsOhc((res + "pc_sample.ohc").c_str())) {
        std::cerr << "Fail to save OHC file" << std::endl;
        return 1;
    }
    Hologram->encoding(Hologram->ENCODE_PHASE);
    Hologram->normalize();
    if (!Hologram->save((res + "pc_sample.bmp").c_str())) {
        std::cerr << "Fail to save BMP file" << std::endl;
        return 1;
    }
    Hologram->release();
    return 0;
}
