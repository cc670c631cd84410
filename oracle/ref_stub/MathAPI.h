// Export macro of the reference Math library (normally generated by CMake's GenerateExportHeader).
#pragma once
#define MATH_EXPORT
