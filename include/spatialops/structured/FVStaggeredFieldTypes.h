// Field typedefs of the staggered finite-volume mesh and the face types of each volume
// (drop-in for spatialops/structured/FVStaggeredFieldTypes.h:148-217).
#ifndef SpatialOps_FVStaggeredFieldTypes_h
#define SpatialOps_FVStaggeredFieldTypes_h

#include <spatialops/structured/FVStaggeredLocationTypes.h>
#include <spatialops/structured/SpatialField.h>

namespace SpatialOps {

typedef SpatialField<SVol> SVolField;
typedef SpatialField<SSurfX> SSurfXField;
typedef SpatialField<SSurfY> SSurfYField;
typedef SpatialField<SSurfZ> SSurfZField;
typedef SpatialField<XVol> XVolField;
typedef SpatialField<XSurfX> XSurfXField;
typedef SpatialField<XSurfY> XSurfYField;
typedef SpatialField<XSurfZ> XSurfZField;
typedef SpatialField<YVol> YVolField;
typedef SpatialField<YSurfX> YSurfXField;
typedef SpatialField<YSurfY> YSurfYField;
typedef SpatialField<YSurfZ> YSurfZField;
typedef SpatialField<ZVol> ZVolField;
typedef SpatialField<ZSurfX> ZSurfXField;
typedef SpatialField<ZSurfY> ZSurfYField;
typedef SpatialField<ZSurfZ> ZSurfZField;
// one value held in a field (a 1x1x1 window without ghosts); broadcast where it meets a field
typedef SpatialField<SingleValue> SingleValueField;

template <typename VolT> struct FaceTypes;
template <> struct FaceTypes<SVolField> { typedef SSurfXField XFace; typedef SSurfYField YFace; typedef SSurfZField ZFace; };
template <> struct FaceTypes<XVolField> { typedef XSurfXField XFace; typedef XSurfYField YFace; typedef XSurfZField ZFace; };
template <> struct FaceTypes<YVolField> { typedef YSurfXField XFace; typedef YSurfYField YFace; typedef YSurfZField ZFace; };
template <> struct FaceTypes<ZVolField> { typedef ZSurfXField XFace; typedef ZSurfYField YFace; typedef ZSurfZField ZFace; };

template <typename FaceT> struct VolType;
template <> struct VolType<SSurfXField> { typedef SVolField VolField; };
template <> struct VolType<SSurfYField> { typedef SVolField VolField; };
template <> struct VolType<SSurfZField> { typedef SVolField VolField; };
template <> struct VolType<XSurfXField> { typedef XVolField VolField; };
template <> struct VolType<XSurfYField> { typedef XVolField VolField; };
template <> struct VolType<XSurfZField> { typedef XVolField VolField; };
template <> struct VolType<YSurfXField> { typedef YVolField VolField; };
template <> struct VolType<YSurfYField> { typedef YVolField VolField; };
template <> struct VolType<YSurfZField> { typedef YVolField VolField; };
template <> struct VolType<ZSurfXField> { typedef ZVolField VolField; };
template <> struct VolType<ZSurfYField> { typedef ZVolField VolField; };
template <> struct VolType<ZSurfZField> { typedef ZVolField VolField; };

}  // namespace SpatialOps
#endif
