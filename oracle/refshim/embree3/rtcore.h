// Declarations of the Embree 3 names that CRender's entity header
// (src/render/entities/components.h) mentions, so that the header compiles for
// the oracle's cross-check; none of them is defined or called there.
// TEST INFRASTRUCTURE ONLY.
#pragma once
typedef struct RTCDeviceTy *RTCDevice;
typedef struct RTCSceneTy *RTCScene;
typedef struct RTCGeometryTy *RTCGeometry;
enum RTCGeometryType { RTC_GEOMETRY_TYPE_TRIANGLE = 0 };
RTCDevice rtcNewDevice(const char *config);
RTCScene rtcNewScene(RTCDevice device);
RTCGeometry rtcNewGeometry(RTCDevice device, enum RTCGeometryType type);
