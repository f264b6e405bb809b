// Stand-in for <windows.h> when compiling the reference's src/octree/Rle4.cpp
// for the host (TEST INFRASTRUCTURE ONLY): Rle4.cpp only calls MessageBox,
// on a missing file, right before exit(0); the caller checks the file first.
#pragma once
#define MessageBox(owner, text, caption, type) 0
