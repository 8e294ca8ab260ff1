// Minimal assimp scene types: enough for the reference's load code to compile.
#pragma once
struct aiString { const char *C_Str() const { return ""; } };
struct aiVector3D { float x, y, z; };
struct aiFace { unsigned int mNumIndices; unsigned int *mIndices; };
enum aiPrimitiveType { aiPrimitiveType_TRIANGLE = 4 };
struct aiMesh {
  unsigned int mPrimitiveTypes, mNumVertices, mNumFaces;
  aiVector3D *mVertices;
  aiFace *mFaces;
  aiString mName;
  bool HasFaces() const { return mNumFaces > 0; }
};
struct aiMatrix4x4 { float a1, a2, a3, a4, b1, b2, b3, b4, c1, c2, c3, c4, d1, d2, d3, d4; };
struct aiNode { unsigned int mNumChildren; aiMatrix4x4 mTransformation; };
struct aiScene {
  aiNode *mRootNode;
  unsigned int mNumMeshes;
  aiMesh **mMeshes;
  bool HasMeshes() const { return mNumMeshes > 0; }
};
