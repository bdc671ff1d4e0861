// Host-side scene ingest shared between the image decoder (fr_image_read.cpp)
// and the OBJ/MTL loader (fr_ingest.cpp).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace fr {

// An image as TextureUtility::LoadTextureFromFile holds it
// (TextureUtility.cpp:12-35): `channels` is the count stb_image reports with
// req_comp 0; `rgba` has width*height*4 bytes, the file's channels in order
// and the missing ones 0 (alpha 255).
struct DecodedImage {
  int32_t width = 0, height = 0, channels = 0;
  std::vector<uint8_t> rgba;
};

// Decodes an image file; returns "" on success, else the reason.
std::string decode_image_file(const std::string& path, DecodedImage* out);

// Sets the message fr_last_error() returns on this thread; returns code.
int set_last_error(int code, const std::string& message);

}  // namespace fr
