// No-op OutputFile bodies so the PV2013 reference compiles without libvtk
// (OutputFile.cpp:16-137 writes .vtu files only; nothing on the step path
// reads them).  TEST INFRASTRUCTURE ONLY.
#include "OutputFile.h"

OutputFile::OutputFile(int outputIdx) : m_outputIdx(outputIdx) {}
OutputFile::~OutputFile() {}
void OutputFile::WriteVTK_LocalData(SubDomain&) {}
void OutputFile::WriteWallShearStressVTK(SubDomain&, int) {}
